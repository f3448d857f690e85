// field_oracle.cpp -- CPU restatement of the grid sampling of a solve's fields.
//
// TEST INFRASTRUCTURE ONLY: the checker the device sampler (k_grid_claim / k_grid_eval) is
// compared against.  Built with -ffp-contract=off, so every product and sum rounds on its
// own as on the device, and the owners and values agree bit for bit.
//
// The grid is ScalarField_Grid's (include/PhySim/Geometry/Volumes/ScalarField_Grid.h):
// value (i, j, k) at i + s0 * (j + s1 * k), for the cell centre
// origin + (i + 1/2, j + 1/2, k + 1/2) * delta (its Sample method's coordinates).  A centre
// belongs to the lowest-index tet whose four sub-volumes at that centre are each >= -1e-12 of
// the tet's own; the field there is the displacement u = x - X0 interpolated with the
// barycentric weights, its norm, det F, or the element energy over the rest volume.
// This routine visits every (tet, cell of the tet's bounding box) pair, serially.
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct V3 {
  double x, y, z;
};

V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

double det3v(V3 u, V3 v, V3 w) {
  double cx = v.y * w.z - v.z * w.y;
  double cy = v.z * w.x - v.x * w.z;
  double cz = v.x * w.y - v.y * w.x;
  return (u.x * cx + u.y * cy) + u.z * cz;
}

V3 node(const double* X, int v) { return {X[3 * (size_t)v], X[3 * (size_t)v + 1], X[3 * (size_t)v + 2]}; }

void sub_volumes(const V3 X[4], V3 p, double V[4]) {
  const V3 e1 = sub(X[1], X[0]), e2 = sub(X[2], X[0]), e3 = sub(X[3], X[0]), q = sub(p, X[0]);
  V[0] = det3v(sub(X[1], p), sub(X[2], p), sub(X[3], p));
  V[1] = det3v(q, e2, e3);
  V[2] = det3v(e1, q, e3);
  V[3] = det3v(e1, e2, q);
}

double centre(double o, int i, double d) { return o + ((double)i + 0.5) * d; }

bool axis_range(double a, double b, double o, double d, int s, int* lo, int* hi) {
  double ca = (((a - o) / d) - 0.5) - 1e-9;
  double cb = (((b - o) / d) - 0.5) + 1e-9;
  ca = std::fmax(std::ceil(ca), 0.0);
  cb = std::fmin(std::floor(cb), (double)(s - 1));
  if (!(ca <= cb)) return false;
  *lo = (int)ca;
  *hi = (int)cb;
  return true;
}

}  // namespace

extern "C" {

// X0, x: [3n]; T: [4m]; E: [m] element energies (field 5) or NULL; values, owner: [cells].
int orc_sample_grid(int32_t n, int32_t m, const double* X0, const int32_t* T, const double* x, const double* E,
                    int32_t field, const int32_t shape[3], const double origin[3], const double delta[3], double fill,
                    double* values, int32_t* owner) {
  (void)n;
  if (field < 0 || field > 5 || (field == 5 && !E)) return -1;
  const int64_t s0 = shape[0], s1 = shape[1], count = s0 * s1 * shape[2];
  const int32_t none = 0x7fffffff;
  for (int64_t c = 0; c < count; ++c) owner[c] = none;
  for (int e = 0; e < m; ++e) {
    V3 X[4];
    for (int q = 0; q < 4; ++q) X[q] = node(X0, T[4 * (size_t)e + q]);
    const double D = det3v(sub(X[1], X[0]), sub(X[2], X[0]), sub(X[3], X[0]));
    const double tol = -1e-12 * D;
    int lo[3], hi[3];
    double mn[3] = {std::fmin(std::fmin(X[0].x, X[1].x), std::fmin(X[2].x, X[3].x)),
                    std::fmin(std::fmin(X[0].y, X[1].y), std::fmin(X[2].y, X[3].y)),
                    std::fmin(std::fmin(X[0].z, X[1].z), std::fmin(X[2].z, X[3].z))};
    double mx[3] = {std::fmax(std::fmax(X[0].x, X[1].x), std::fmax(X[2].x, X[3].x)),
                    std::fmax(std::fmax(X[0].y, X[1].y), std::fmax(X[2].y, X[3].y)),
                    std::fmax(std::fmax(X[0].z, X[1].z), std::fmax(X[2].z, X[3].z))};
    bool any = true;
    for (int d = 0; d < 3; ++d) any = any && axis_range(mn[d], mx[d], origin[d], delta[d], shape[d], &lo[d], &hi[d]);
    if (!any) continue;
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const V3 p = {centre(origin[0], i, delta[0]), centre(origin[1], j, delta[1]), centre(origin[2], k, delta[2])};
          double V[4];
          sub_volumes(X, p, V);
          if (V[0] >= tol && V[1] >= tol && V[2] >= tol && V[3] >= tol) {
            int32_t& o = owner[i + s0 * (j + s1 * (int64_t)k)];
            if (e < o) o = e;
          }
        }
  }
  for (int64_t c = 0; c < count; ++c) {
    const int e = owner[c];
    if (e == none) {
      owner[c] = -1;
      values[c] = fill;
      continue;
    }
    const int i = (int)(c % s0), j = (int)((c / s0) % s1), k = (int)(c / (s0 * s1));
    const int32_t* t = T + 4 * (size_t)e;
    V3 X[4];
    for (int q = 0; q < 4; ++q) X[q] = node(X0, t[q]);
    const double D = det3v(sub(X[1], X[0]), sub(X[2], X[0]), sub(X[3], X[0]));
    if (field == 4) {
      V3 y[4];
      for (int q = 0; q < 4; ++q) y[q] = node(x, t[q]);
      values[c] = det3v(sub(y[1], y[0]), sub(y[2], y[0]), sub(y[3], y[0])) / D;
      continue;
    }
    if (field == 5) {
      values[c] = E[e] / (D / 6.0);
      continue;
    }
    const V3 p = {centre(origin[0], i, delta[0]), centre(origin[1], j, delta[1]), centre(origin[2], k, delta[2])};
    double V[4];
    sub_volumes(X, p, V);
    const double S = (V[0] + V[1]) + (V[2] + V[3]);
    double u[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 4; ++q) {
      const double w = V[q] / S;
      const V3 dq = sub(node(x, t[q]), X[q]);
      u[0] = u[0] + w * dq.x;
      u[1] = u[1] + w * dq.y;
      u[2] = u[2] + w * dq.z;
    }
    values[c] = field < 3 ? u[field] : std::sqrt((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
  }
  return 0;
}

}  // extern "C"
