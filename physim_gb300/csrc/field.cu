// field.cu -- fields of a solve sampled on a regular grid (field output next to the solve).
//
// ScalarField_Grid (include/PhySim/Geometry/Volumes/ScalarField_Grid.h) places value (i, j, k)
// at the cell centre origin + (i + 1/2, j + 1/2, k + 1/2) * delta (its Sample method maps a
// point p to (p - origin) / delta - 1/2).  These kernels fill such a grid from an instance's
// tets over the rest shape:
//
//   k_grid_init   every cell: owner = none
//   k_grid_claim  one warp per tet: the lanes walk the cells whose centres lie in the tet's
//                 bounding box and claim each centre the tet contains (atomicMin of the tet
//                 index: the lowest index wins where tets share a face, edge or node)
//   k_grid_eval   one thread per cell: the owning tet's barycentric weights at the centre
//                 and the field there (displacement interpolated from the four corners,
//                 det F or energy density of the tet), `fill` where no tet owns the centre
//
// Containment: the four signed volumes a centre p cuts the tet (X0..X3) into, each computed
// as a 3x3 determinant of edge vectors, are >= -1e-12 of the tet's own.  Every product and
// sum below is an explicitly rounded operation (no contraction into fused multiply-adds), so
// a CPU restatement of the same steps gives the same owners and the same bits.
#include <cstdint>

#include "kernels.h"

namespace phx {
namespace {

constexpr int kNoOwner = 0x7fffffff;
constexpr double kInsideTol = 1e-12;
constexpr double kRangeSlack = 1e-9;  // cells tested beyond the bounding box (index units)

struct V3 {
  double x, y, z;
};

__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }

// u . (v x w), in a fixed order of rounded operations
__device__ __forceinline__ double det3v(V3 u, V3 v, V3 w) {
  double cx = __dsub_rn(__dmul_rn(v.y, w.z), __dmul_rn(v.z, w.y));
  double cy = __dsub_rn(__dmul_rn(v.z, w.x), __dmul_rn(v.x, w.z));
  double cz = __dsub_rn(__dmul_rn(v.x, w.y), __dmul_rn(v.y, w.x));
  return __dadd_rn(__dadd_rn(__dmul_rn(u.x, cx), __dmul_rn(u.y, cy)), __dmul_rn(u.z, cz));
}

__device__ __forceinline__ V3 node(const double* xs, int v) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(xs + 4 * (size_t)v));
  const double b = __ldg(xs + 4 * (size_t)v + 2);
  return {a.x, a.y, b};
}

// Signed volumes (times six) of the sub-tets p X1 X2 X3, X0 p X2 X3, X0 X1 p X3, X0 X1 X2 p.
__device__ __forceinline__ void sub_volumes(const V3 X[4], V3 p, double V[4]) {
  const V3 e1 = sub(X[1], X[0]), e2 = sub(X[2], X[0]), e3 = sub(X[3], X[0]), q = sub(p, X[0]);
  V[0] = det3v(sub(X[1], p), sub(X[2], p), sub(X[3], p));
  V[1] = det3v(q, e2, e3);
  V[2] = det3v(e1, q, e3);
  V[3] = det3v(e1, e2, q);
}

__device__ __forceinline__ double centre(double o, int i, double d) {
  return __dadd_rn(o, __dmul_rn(__dadd_rn((double)i, 0.5), d));
}

// Cells [lo, hi] of one axis whose centres may lie in [a, b].
__device__ __forceinline__ void axis_range(double a, double b, double o, double d, int s, int* lo, int* hi) {
  double ca = __dsub_rn(__dsub_rn(__ddiv_rn(__dsub_rn(a, o), d), 0.5), kRangeSlack);
  double cb = __dadd_rn(__dsub_rn(__ddiv_rn(__dsub_rn(b, o), d), 0.5), kRangeSlack);
  ca = fmax(ceil(ca), 0.0);
  cb = fmin(floor(cb), (double)(s - 1));
  if (!(ca <= cb)) {
    *lo = 1;
    *hi = 0;
    return;
  }
  *lo = (int)ca;
  *hi = (int)cb;
}

__global__ void k_grid_init(int32_t* owner, int64_t count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    owner[i] = kNoOwner;
}

__global__ void __launch_bounds__(256) k_grid_claim(GridSampleArgs a) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < a.m; e += warps) {
    const int4 t = __ldg(reinterpret_cast<const int4*>(a.tets) + e);
    const V3 X[4] = {node(a.xrest, t.x), node(a.xrest, t.y), node(a.xrest, t.z), node(a.xrest, t.w)};
    const double D = det3v(sub(X[1], X[0]), sub(X[2], X[0]), sub(X[3], X[0]));
    const double tol = __dmul_rn(-kInsideTol, D);
    int lo[3], hi[3];
    axis_range(fmin(fmin(X[0].x, X[1].x), fmin(X[2].x, X[3].x)), fmax(fmax(X[0].x, X[1].x), fmax(X[2].x, X[3].x)),
               a.origin[0], a.delta[0], a.shape[0], &lo[0], &hi[0]);
    axis_range(fmin(fmin(X[0].y, X[1].y), fmin(X[2].y, X[3].y)), fmax(fmax(X[0].y, X[1].y), fmax(X[2].y, X[3].y)),
               a.origin[1], a.delta[1], a.shape[1], &lo[1], &hi[1]);
    axis_range(fmin(fmin(X[0].z, X[1].z), fmin(X[2].z, X[3].z)), fmax(fmax(X[0].z, X[1].z), fmax(X[2].z, X[3].z)),
               a.origin[2], a.delta[2], a.shape[2], &lo[2], &hi[2]);
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) continue;
    const int64_t ni = hi[0] - lo[0] + 1, nj = hi[1] - lo[1] + 1, nk = hi[2] - lo[2] + 1;
    const int64_t cells = ni * nj * nk;
    for (int64_t c = lane; c < cells; c += 32) {
      const int i = lo[0] + (int)(c % ni), j = lo[1] + (int)((c / ni) % nj), k = lo[2] + (int)(c / (ni * nj));
      const V3 p = {centre(a.origin[0], i, a.delta[0]), centre(a.origin[1], j, a.delta[1]),
                    centre(a.origin[2], k, a.delta[2])};
      double V[4];
      sub_volumes(X, p, V);
      if (V[0] >= tol && V[1] >= tol && V[2] >= tol && V[3] >= tol)
        atomicMin(a.owner + (i + (int64_t)a.shape[0] * (j + (int64_t)a.shape[1] * k)), e);
    }
  }
}

__global__ void k_grid_eval(GridSampleArgs a) {
  const int64_t count = (int64_t)a.shape[0] * a.shape[1] * a.shape[2];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < count; c += (int64_t)gridDim.x * blockDim.x) {
    const int e = a.owner[c];
    if (e == kNoOwner) {
      a.owner[c] = -1;
      a.values[c] = a.fill;
      continue;
    }
    const int i = (int)(c % a.shape[0]), j = (int)((c / a.shape[0]) % a.shape[1]),
              k = (int)(c / ((int64_t)a.shape[0] * a.shape[1]));
    const int4 t = __ldg(reinterpret_cast<const int4*>(a.tets) + e);
    const int ids[4] = {t.x, t.y, t.z, t.w};
    V3 X[4];
    for (int q = 0; q < 4; ++q) X[q] = node(a.xrest, ids[q]);
    const double D = det3v(sub(X[1], X[0]), sub(X[2], X[0]), sub(X[3], X[0]));
    double val;
    if (a.field == 4 || a.field == 5) {
      if (a.field == 4) {
        V3 x[4];
        for (int q = 0; q < 4; ++q) x[q] = node(a.x, ids[q]);
        val = __ddiv_rn(det3v(sub(x[1], x[0]), sub(x[2], x[0]), sub(x[3], x[0])), D);
      } else {
        val = __ddiv_rn(a.energy[e], __ddiv_rn(D, 6.0));
      }
    } else {
      const V3 p = {centre(a.origin[0], i, a.delta[0]), centre(a.origin[1], j, a.delta[1]),
                    centre(a.origin[2], k, a.delta[2])};
      double V[4];
      sub_volumes(X, p, V);
      const double S = __dadd_rn(__dadd_rn(V[0], V[1]), __dadd_rn(V[2], V[3]));
      double u[3] = {0.0, 0.0, 0.0};
      for (int q = 0; q < 4; ++q) {
        const double w = __ddiv_rn(V[q], S);
        const V3 xq = node(a.x, ids[q]);
        const V3 dq = sub(xq, X[q]);
        u[0] = __dadd_rn(u[0], __dmul_rn(w, dq.x));
        u[1] = __dadd_rn(u[1], __dmul_rn(w, dq.y));
        u[2] = __dadd_rn(u[2], __dmul_rn(w, dq.z));
      }
      if (a.field < 3)
        val = u[a.field];
      else
        val = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(u[0], u[0]), __dmul_rn(u[1], u[1])), __dmul_rn(u[2], u[2])));
    }
    a.values[c] = val;
  }
}

}  // namespace

cudaError_t launch_grid_sample(cudaStream_t s, const GridSampleArgs& a, int num_sms) {
  const int64_t count = (int64_t)a.shape[0] * a.shape[1] * a.shape[2];
  const int cells_grid = (int)std::min<int64_t>((count + 255) / 256, 8 * (int64_t)num_sms);
  k_grid_init<<<cells_grid, 256, 0, s>>>(a.owner, count);
  const int tet_grid = (int)std::min<int64_t>(((int64_t)a.m + 7) / 8, 32 * (int64_t)num_sms);
  if (tet_grid > 0) k_grid_claim<<<tet_grid, 256, 0, s>>>(a);
  k_grid_eval<<<cells_grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace phx
