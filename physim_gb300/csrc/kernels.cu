// kernels.cu -- sm_103a kernels of the tet-FEM Newton path.
//
// Every kernel is persistent over a packed tile index of the active batch:
// tiles of 128 tets, 128 nodes (4 SELL chunks of 32 rows) or 128 lower blocks,
// numbered instance by instance through prefix arrays, so uneven meshes share
// one launch.  A kernel touches only the instances whose Newton state is in
// the phase it serves; the others' tiles are skipped.  Per-instance reductions
// are deterministic: each tile writes its partial sums, and the CTA that
// finishes an instance's last tile (counted with one atomic) sums the partials
// in tile order and advances that instance's state.  Nothing waits on another
// CTA, so no kernel here can hang.
//
// Reference behaviour each kernel restates:
//   k_elem_eg     EnergyElement_FEM::ComputeAndStore_{Energy,Gradient}_Internal
//                 (source/PhySim/Physics/Elements/EnergyElement_FEM.cpp:125-191),
//                 inverted element -> energy HUGE_VAL (:126-131)
//   k_gather      Simulable::AddGradient / AddEnergy order (Simulable.cpp:321-521),
//                 lumped-mass gravity (MassElement_Lumped.cpp:56-76), nodal forces
//                 (EnergyElement_Force.cpp:43-56), FixVectorDoFs (Simulable.cpp:735-744),
//                 implicit-Euler inertia (OptimProblem_BasicDynamic.cpp:58-101)
//   k_elem_hess   EnergyElement_FEM::ComputeAndStore_Hessian_Internal (:193-222)
//   k_assemble    DerivativeAssembler::AssembleHessian + AMatrixSd static blocks
//                 (DerivativeAssembler.cpp:268-300, BasicTypes.cpp:45-62) and
//                 FixMatrixDoFs (Simulable.cpp:746-760); + M/dt^2 for dynamics
//   k_jacobi ... k_accum   LinearSolver_EigenCG::SolveInternal (LinearSolver_EigenCG.cpp:51-125)
//                 with a 3x3 block-Jacobi (or Eigen's diagonal) preconditioner and,
//                 on the FP32 path, FP64 residual refinement sweeps.
#include <cfloat>
#include <cstdint>
#include <algorithm>
#include <type_traits>

#include "element.cuh"
#include "kernels.h"
#include "newton_control.h"

namespace phx {

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tiles_of(int count) { return (count + kTile - 1) / kTile; }
// PCG tiles of an instance: one SELL chunk (32 rows) per tile up to kOneChunkTiles chunks, so
// that a small instance iterating alone spreads over many CTAs; four chunks (128 rows, one per
// thread) above.  The width is the instance's own, so its per-tile partial sums, and with them
// its bits, do not depend on the batch it runs in.
__device__ __forceinline__ int pcg_cpt(const InstDev& I) { return I.nchunks <= kOneChunkTiles ? 1 : 4; }
__device__ __forceinline__ int pcg_tiles(const BatchDev&, const InstDev& I) {
  const int cpt = pcg_cpt(I);
  return (I.nchunks + cpt - 1) / cpt;
}
// true when this instance's PCG is left to the cluster kernel in this launch
__device__ __forceinline__ bool cluster_owned(const BatchDev& B, const InstDev& I) {
  return B.cluster_mode && I.pcg_cluster;
}

// Sums K values over the CTA into v[] of warp 0 (fixed order); T = double, or float for
// the FP32 PCG's per-tile inner products (sm: the double scratch, reused as T).
template <int K, typename T = double>
__device__ __forceinline__ void block_sum(T (&v)[K], double* smd) {
  T* sm = reinterpret_cast<T*>(smd);
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sm[warp * K + k] = v[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      v[k] = lane < nw ? sm[lane * K + k] : (T)0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    }
  }
}

// tile_done without a reduction: for stages that only need to know which CTA completes the
// instance (the same one-atomic-per-CTA count).  Returns true in that CTA (all threads).
__device__ __forceinline__ bool tile_count_done(const InstDev& I, int lt, int ntiles, int ncta, int* flag) {
  if (lt + ncta < ntiles) return false;  // not this CTA's last tile of the instance
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned mine = (unsigned)(lt / ncta + 1);
    __threadfence();
    const unsigned prev = atomicAdd(I.counter, mine);
    *flag = (prev + mine == (unsigned)ntiles);
    if (*flag) *I.counter = 0u;
  }
  __syncthreads();
  if (!*flag) return false;
  __threadfence();
  return true;
}

__device__ __forceinline__ void count_bytes(const BatchDev& B, const InstDev& I, KernelId k) {
  if (B.algo_total) B.algo_total[k] += I.algo[k];  // single thread of the finalising CTA
}

// Records this tile's partial sums; in the CTA that completes the instance's last tile,
// returns true and leaves the instance totals in thread 0's tot[].  Tiles are dealt to the
// ncta CTAs round-robin (t = cta, cta + ncta, ...), and the instance's tiles are
// contiguous, so a CTA's last tile of the instance is the one with lt + ncta >= ntiles and
// it has then done lt / ncta + 1 of them: only that tile publishes the count, with one
// fence and one atomic per CTA and instance instead of per tile.  The totals are summed
// from the per-tile partials in tile order, whatever the CTA count.
template <int K, typename T>
__device__ bool tile_done(const InstDev& I, int lt, int ntiles, int ncta, T (&v)[K], double (&tot)[K],
                          double* sm, int* flag) {
  block_sum<K, T>(v, sm);
  const bool last_here = lt + ncta >= ntiles;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) I.partials[(size_t)lt * K + k] = (double)v[k];
    if (last_here) {
      const unsigned mine = (unsigned)(lt / ncta + 1);
      __threadfence();
      const unsigned prev = atomicAdd(I.counter, mine);
      *flag = (prev + mine == (unsigned)ntiles);
    }
  }
  if (!last_here) return false;
  __syncthreads();
  if (!*flag) return false;
  __threadfence();
  // four independent running sums per thread (tiles t, t + bd, t + 2 bd, t + 3 bd) keep
  // four loads in flight: an instance with thousands of tiles is summed by one CTA while
  // the others wait at the next barrier.  The order depends on the tile count only.
  double acc[K], a1[K], a2[K], a3[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = a1[k] = a2[k] = a3[k] = 0.0;
  const int bd = blockDim.x;
  int t = threadIdx.x;
  for (; t + 3 * bd < ntiles; t += 4 * bd)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      acc[k] += __ldcg(I.partials + (size_t)t * K + k);
      a1[k] += __ldcg(I.partials + (size_t)(t + bd) * K + k);
      a2[k] += __ldcg(I.partials + (size_t)(t + 2 * bd) * K + k);
      a3[k] += __ldcg(I.partials + (size_t)(t + 3 * bd) * K + k);
    }
  for (; t < ntiles; t += bd)
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] += __ldcg(I.partials + (size_t)t * K + k);
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = (acc[k] + a1[k]) + (a2[k] + a3[k]);
  block_sum<K>(acc, sm);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) tot[k] = acc[k];
    *I.counter = 0u;
  }
  return true;
}

__device__ __forceinline__ void ld4(const double* p, int64_t v, double (&o)[3]) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * v;
  double2 a = q[0], b = q[1];
  o[0] = a.x; o[1] = a.y; o[2] = b.x;
}
__device__ __forceinline__ void st4(double* p, int64_t v, const double (&o)[3]) {
  double2* q = reinterpret_cast<double2*>(p) + 2 * v;
  q[0] = make_double2(o[0], o[1]);
  q[1] = make_double2(o[2], 0.0);
}
__device__ __forceinline__ void ld4(const float* p, int64_t v, float (&o)[3]) {
  float4 a = reinterpret_cast<const float4*>(p)[v];
  o[0] = a.x; o[1] = a.y; o[2] = a.z;
}
__device__ __forceinline__ void st4(float* p, int64_t v, const float (&o)[3]) {
  reinterpret_cast<float4*>(p)[v] = make_float4(o[0], o[1], o[2], 0.f);
}

template <typename T> struct PcgBufs;
template <> struct PcgBufs<float> {
  __device__ static float* H(const InstDev& I) { return I.H32; }
  __device__ static float* Hloc(const InstDev& I) { return I.Hloc32; }
  __device__ static float* r(const InstDev& I) { return I.r32; }
  __device__ static float* z(const InstDev& I) { return I.z32; }
  __device__ static float* pa(const InstDev& I) { return I.p32a; }
  __device__ static float* pb(const InstDev& I) { return I.p32b; }
  __device__ static float* q(const InstDev& I) { return I.q32; }
  __device__ static float* e(const InstDev& I) { return I.e32; }
  __device__ static float* minv(const InstDev& I) { return I.minv32; }
  __device__ static const float* rest(const InstDev& I) { return I.rest32; }
};
template <> struct PcgBufs<double> {
  __device__ static double* H(const InstDev& I) { return I.H64; }
  __device__ static double* Hloc(const InstDev& I) { return I.Hloc64; }
  __device__ static double* r(const InstDev& I) { return I.rd; }
  __device__ static double* z(const InstDev& I) { return I.zd; }
  __device__ static double* pa(const InstDev& I) { return I.pda; }
  __device__ static double* pb(const InstDev& I) { return I.pdb; }
  __device__ static double* q(const InstDev& I) { return I.qd; }
  __device__ static double* e(const InstDev& I) { return I.ed; }
  __device__ static double* minv(const InstDev& I) { return I.minvd; }
  __device__ static const double* rest(const InstDev& I) { return I.rest64; }
};

// Loads a tet's displacement differences Du = [u1-u0, u2-u0, u3-u0], u = x - X0, in FP64.
// F - I = Du Dm^-1 then carries no cancellation against the rest shape, so small strains
// keep their digits in the strain measures below.
__device__ __forceinline__ void load_du(const InstDev& I, int e, int (&nd)[4], double (&Du)[9]) {
  int4 t = reinterpret_cast<const int4*>(I.tets)[e];
  nd[0] = t.x; nd[1] = t.y; nd[2] = t.z; nd[3] = t.w;
  double u0[3], ua[3], X[3];
  ld4(I.x, nd[0], u0);
  ld4(I.xrest, nd[0], X);
  for (int r = 0; r < 3; ++r) u0[r] -= X[r];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    ld4(I.x, nd[c + 1], ua);
    ld4(I.xrest, nd[c + 1], X);
#pragma unroll
    for (int r = 0; r < 3; ++r) Du[r + 3 * c] = (ua[r] - X[r]) - u0[r];
  }
}

// y - log(1 + y) without cancellation for small y (series up to y^9 when |y| < 1e-3)
// y - log1p(y) without cancellation; l1p = log1p(y), already computed by the caller.  For
// |y| < 1e-3 the series sum_{k>=2} (-1)^k y^k / k, in Horner form with the coefficients as
// constants (no FP64 divisions), truncated after y^9 (relative error below 1e-24 there).
__device__ __forceinline__ double y_minus_log1p(double y, double l1p) {
  if (fabs(y) < 1e-3) {
    double s = 1.0 / 9.0;
    s = 1.0 / 8.0 - y * s;
    s = 1.0 / 7.0 - y * s;
    s = 1.0 / 6.0 - y * s;
    s = 1.0 / 5.0 - y * s;
    s = 1.0 / 4.0 - y * s;
    s = 1.0 / 3.0 - y * s;
    s = 1.0 / 2.0 - y * s;
    return (y * y) * s;
  }
  return y - l1p;
}

// ---------------------------------------------------------------------------
// tile maps: a list of instances (all of a batch, or the compacted active ones)
// and the prefix of their tile counts.  Loaded through L2 (ld.cg) because the
// engine rewrites them between rounds inside one launch.
// ---------------------------------------------------------------------------
struct TileMap {
  const int32_t* pre;  // [num + 1]
  const int32_t* ids;  // [num] list entry -> instance, or null for the identity
  int num;
};

__device__ __forceinline__ int map_total(const TileMap& M) { return __ldcg(M.pre + M.num); }

__device__ __forceinline__ void map_tile(const TileMap& M, int t, int& inst, int& lt) {
  int lo = 0, hi = M.num;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldcg(M.pre + mid) <= t) lo = mid; else hi = mid;
  }
  inst = M.ids ? __ldcg(M.ids + lo) : lo;
  lt = t - __ldcg(M.pre + lo);
}

__device__ __forceinline__ TileMap full_map(const BatchDev& B, const int32_t* pre) {
  return TileMap{pre, nullptr, *B.num};
}

// Runs the state machine of instance i up to its next device phase (called by the one
// thread that finalises a stage for the instance) and publishes the phase.
// Phase bucket of an instance for the engine's stage counts: its phase, except that a PCG
// solve left to the cluster kernel has a bucket of its own.
__device__ __forceinline__ int phase_bucket(const BatchDev& B, const InstDev& I, int ph) {
  return (ph == PH_PCG && cluster_owned(B, I)) ? kBucketClusterPcg : ph;
}

__device__ void advance(const BatchDev& B, int i) {
  const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
  NState s = *I.st;
  ctl_advance(s, *I.opts);
  if (s.log_pending) {
    if (I.log && s.log_count < kLogCap) {
      I.log[4 * s.log_count + 0] = s.obj;
      I.log[4 * s.log_count + 1] = s.opt;
      I.log[4 * s.log_count + 2] = (double)s.num_bis;
      I.log[4 * s.log_count + 3] = s.log_step;
    }
    s.log_count++;
    s.log_pending = 0;
  }
  *I.st = s;
  if (B.phase_live) {  // move the instance between the per-phase counts the engine skips stages by
    const int old = B.flags[8 + i];
    const int ob = (old > PH_DONE && old < kBucketClusterPcg) ? phase_bucket(B, I, old) : -1;
    const int nb = s.phase > PH_DONE ? phase_bucket(B, I, s.phase) : -1;
    if (ob != nb) {
      if (ob >= 0) atomicSub(B.phase_live + ob, 1);
      if (nb >= 0) atomicAdd(B.phase_live + nb, 1);
    }
  }
  B.flags[8 + i] = s.phase;
}

// ---------------------------------------------------------------------------
// vector ops of the state machine
// ---------------------------------------------------------------------------
// One node's boundary-condition values at `stage` (BC_FixDoF::Update, BC_FixDoF.cpp:80-121):
// its group's a = min(stage, N) / N; the target a b + (I + a M) v of the start value v
// (VectorAnimator_LerpT3D::Evaluate, VectorAnimators.h:135-145); a hard group's node takes
// it as its position (the static problem: the dynamic one's predictor overwrites positions),
// a soft group's node takes it as its target with the stiffness k0 + a (k1 - k0).  Called on
// the iteration's start state (x = the last accepted iterate).
__device__ __forceinline__ void stage_node(const InstDev& I, int v, int stage, double (&x)[3]) {
  if (!I.stage_grp) return;
  const int g = I.stage_grp[v];
  if (g < 0) return;
  const double* P = I.stage_par + 16 * g;
  const int N = (int)P[0];
  const double a = (double)min(stage, N) / (double)N;
  double u[3], t[3];
  ld4(I.stage_ini, v, u);
#pragma unroll
  for (int r = 0; r < 3; ++r)
    t[r] = a * P[13 + r] + u[r] + a * (P[4 + 3 * r] * u[0] + P[5 + 3 * r] * u[1] + P[6 + 3 * r] * u[2]);
  if (P[1] != 0.0) {
    double* q = I.soft + 4 * (size_t)v;
    q[0] = t[0]; q[1] = t[1]; q[2] = t[2];
    q[3] = P[2] + a * (P[3] - P[2]);
  } else if (!I.opts->dynamic) {
    // the Newton step's start guess, x - x at the last accepted step (OptimSolver.cpp:488),
    // includes the move of the staged DoFs
    double d[3];
    ld4(I.dxprev, v, d);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      d[r] += t[r] - x[r];
      x[r] = t[r];
    }
    st4(I.dxprev, v, d);
    st4(I.x, v, x);
  }
}

__device__ __forceinline__ void st_vecop(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_VEC) continue;
    const int ops = st->vecop;
    const double a = st->alpha_trial, dt = I.opts->dt;
    const int v = lt * kTile + threadIdx.x;
    if (v < I.n) {
      double x[3], xs[3], dx[3], tmp[3], tmp2[3];
      ld4(I.x, v, x);
      if (ops & VO_PRED) {
        double vv[3];
        ld4(I.v, v, vv);
        st4(I.x0, v, x);
        st4(I.v0, v, vv);
        for (int c = 0; c < 3; ++c) x[c] = x[c] + dt * vv[c];
        st4(I.x, v, x);
      }
      if (ops & VO_RESTORE) {
        ld4(I.xs, v, x);
        st4(I.x, v, x);
      }
      if (ops & VO_STAGE) stage_node(I, v, st->stage, x);
      if (ops & (VO_ACCEPT | VO_GCOPY | VO_GNEW)) {
        ld4(I.gn, v, tmp);
        st4(I.g, v, tmp);
      }
      if (ops & VO_ACCEPT) {
        ld4(I.dx, v, dx);
        for (int c = 0; c < 3; ++c) tmp2[c] = a * dx[c];
        st4(I.dxprev, v, tmp2);
      }
      if (ops & VO_GCOPY) st4(I.xback, v, x);  // start of a solve
      if (ops & VO_BACK) {                      // the accepted iterate being left
        ld4(I.xs, v, tmp2);
        st4(I.xback, v, tmp2);
      }
      if (ops & VO_SAVE) st4(I.xs, v, x);
      if (ops & VO_ZERODX) {
        for (int c = 0; c < 3; ++c) tmp[c] = 0.0;
        st4(I.dx, v, tmp);
      }
      if (ops & VO_STEEP) {
        ld4(I.g, v, tmp);
        for (int c = 0; c < 3; ++c) tmp[c] = -tmp[c];
        st4(I.dx, v, tmp);
      }
      if (ops & VO_TRIAL) {
        ld4(I.xs, v, xs);
        ld4(I.dx, v, dx);
        for (int c = 0; c < 3; ++c) x[c] = xs[c] + a * dx[c];
        st4(I.x, v, x);
      }
      if (ops & VO_VEL) {
        double x0[3];
        ld4(I.x0, v, x0);
        for (int c = 0; c < 3; ++c) tmp[c] = (x[c] - x0[c]) / dt;
        st4(I.v, v, tmp);
      }
    }
    if (tile_count_done(I, lt, tiles_of(I.n), ncta, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_VECOP);
      st->phase = st->next_phase;
      st->vecop = 0;
      advance(B, i);
    }
  }
}

// ---------------------------------------------------------------------------
// element energy + gradient (FP64)
// ---------------------------------------------------------------------------
// Energy density and PK1 from the displacement gradient H = F - I (column-major).
// CoNH:  psi = mu/2 (|H|^2 - 2 q + 2 f(j)) + lam/2 log(J)^2, with J - 1 = j = tr H + q,
//        q = I2(H) + det H and f(j) = j - log(1 + j): the same function as
//        mu/2 (tr F^T F - 3 - log J^2) + lam/8 (log J^2)^2 written without cancellation;
//        P = mu F + (lam/2 log J^2 - mu) F^-T.
// StVK:  E = (H + H^T + H^T H)/2, psi = lam/2 tr(E)^2 + mu E:E, P = F (lam tr(E) I + 2 mu E).
__device__ __forceinline__ void material_eg(int model, double lam, double mu, const double* H, double* psi,
                                            double* P, bool* inverted) {
  double F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) F[k] = H[k];
  F[0] += 1.0; F[4] += 1.0; F[8] += 1.0;
  const double trH = H[0] + H[4] + H[8];
  const double I2 = H[0] * H[4] - H[3] * H[1] + H[0] * H[8] - H[6] * H[2] + H[4] * H[8] - H[7] * H[5];
  const double q = I2 + det3(H);
  const double j = trH + q;  // J - 1
  *inverted = j < -1.0;
  if (model == 1) {
    double E[9];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        E[i + 3 * jj] = 0.5 * (H[i + 3 * jj] + H[jj + 3 * i] + H[3 * i] * H[3 * jj] + H[1 + 3 * i] * H[1 + 3 * jj] +
                                H[2 + 3 * i] * H[2 + 3 * jj]);
    double trE = E[0] + E[4] + E[8];
    double ee = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) ee += E[k] * E[k];
    *psi = 0.5 * lam * trE * trE + mu * ee;
    double S[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) S[k] = 2.0 * mu * E[k];
    S[0] += lam * trE; S[4] += lam * trE; S[8] += lam * trE;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
#pragma unroll
      for (int i = 0; i < 3; ++i) P[i + 3 * jj] = F[i] * S[3 * jj] + F[i + 3] * S[1 + 3 * jj] + F[i + 6] * S[2 + 3 * jj];
  } else {
    double hh = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) hh += H[k] * H[k];
    const double J = 1.0 + j;
    const double l1p = (j > -1.0) ? log1p(j) : 0.0;
    const double logJ2 = (j > -1.0) ? 2.0 * l1p : log(J * J);
    const double lJ = 0.5 * logJ2;
    *psi = 0.5 * mu * (hh - 2.0 * q + 2.0 * ((j > -1.0) ? y_minus_log1p(j, l1p) : j - lJ)) + 0.5 * lam * lJ * lJ;
    double C[9];
    cof3(F, C);
    double c = (0.5 * lam * logJ2 - mu) / J;
#pragma unroll
    for (int k = 0; k < 9; ++k) P[k] = mu * F[k] + c * C[k];
  }
}

// EnergyElement_SoftConstraint on one node's ConstraintSet_FixedPosition (BC_FixDoF soft
// mode, EnergyElement_SoftConstraint.cpp:45-86): E = k/2 |x - t|^2, added gradient k (x - t)
// (the Hessian's k I goes to the diagonal block in assembly).
struct SoftNode {
  double t[3], k;
};
__device__ __forceinline__ SoftNode ld_soft(const InstDev& I, int v) {
  SoftNode s{{0.0, 0.0, 0.0}, 0.0};
  if (I.soft) {
    const double2* p = reinterpret_cast<const double2*>(I.soft + 4 * (size_t)v);
    const double2 a = p[0], b = p[1];
    s.t[0] = a.x; s.t[1] = a.y; s.t[2] = b.x; s.k = b.y;
  }
  return s;
}
__device__ __forceinline__ double soft_energy(const SoftNode& s, const double x[3], double* g) {
  const double d[3] = {x[0] - s.t[0], x[1] - s.t[1], x[2] - s.t[2]};
  if (g)
#pragma unroll
    for (int c = 0; c < 3; ++c) g[c] += s.k * d[c];
  return 0.5 * s.k * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

// Node staging of the element stage: a tile's distinct nodes (node lists built with the
// pattern, ascending) are loaded once, coalesced, and their displacements u = x - X0 kept in
// shared memory in FP64; each tet then takes its displacement differences from there
// (Du = u_c - u_0, the same bits as gathering the four corners).
constexpr int kTileNodeCap = 4 * kTile;  // distinct nodes of a tile, at most

// Stages u = x - X0 (x given per node by the functor) of the tile's distinct nodes into
// shared memory, [3][kTileNodeCap] doubles; returns the node count.  Ends with a barrier.
template <typename GetX>
__device__ __forceinline__ int stage_nodes(const InstDev& I, int lt, double* U, GetX getx) {
  const int p0 = __ldg(I.tile_nptr + lt), cnt = __ldg(I.tile_nptr + lt + 1) - p0;
  __syncthreads();  // the previous tile's readers are done with U
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
    const int v = __ldg(I.tile_nodes + p0 + k);
    double x[3], X[3];
    getx(v, x);
    ld4(I.xrest, v, X);
#pragma unroll
    for (int r = 0; r < 3; ++r) U[r * kTileNodeCap + k] = x[r] - X[r];
  }
  __syncthreads();
  return cnt;
}

// Displacement differences of tet e from the staged nodes.
__device__ __forceinline__ void staged_du(const InstDev& I, int e, const double* U, double (&Du)[9]) {
  const ushort4 lc = reinterpret_cast<const ushort4*>(I.tet_loc)[e];
  const int loc[4] = {lc.x, lc.y, lc.z, lc.w};
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) Du[r + 3 * c] = U[r * kTileNodeCap + loc[c + 1]] - U[r * kTileNodeCap + loc[0]];
}

__device__ __forceinline__ void st_elem_eg(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag,
                                           unsigned char* smraw) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_EVAL) continue;
    const int e = lt * kTile + threadIdx.x;
    double Ee = 0.0;
    double* U = reinterpret_cast<double*>(smraw);
    stage_nodes(I, lt, U, [&](int v, double (&x)[3]) { ld4(I.x, v, x); });
    if (e < I.m) {
      double Du[9];
      staged_du(I, e, U, Du);
      double R[12];
      const double2* r2 = reinterpret_cast<const double2*>(I.rest64 + 12 * (size_t)e);
#pragma unroll
      for (int k = 0; k < 6; ++k) { double2 q = r2[k]; R[2 * k] = q.x; R[2 * k + 1] = q.y; }
      double Hd[9];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          Hd[r + 3 * c] = Du[r] * R[0 + 3 * c] + Du[r + 3] * R[1 + 3 * c] + Du[r + 6] * R[2 + 3 * c];
      const double w = R[9], lam = R[10], mu = R[11];
      double psi, P[9];
      bool inverted;
      material_eg(I.model[e], lam, mu, Hd, &psi, P, &inverted);
      Ee = inverted ? __longlong_as_double(0x7ff0000000000000LL) : psi * w;
      // g_a = w * P * B_a, B_a = row (a-1) of Dm^-1, B_0 = -(B_1 + B_2 + B_3)
      double g[12];
#pragma unroll
      for (int a = 1; a < 4; ++a)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          g[3 * a + r] = (P[r] * R[(a - 1)] + P[r + 3] * R[(a - 1) + 3] + P[r + 6] * R[(a - 1) + 6]) * w;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        double b0 = -(R[0] + R[1] + R[2]), b1 = -(R[3] + R[4] + R[5]), b2 = -(R[6] + R[7] + R[8]);
        g[r] = (P[r] * b0 + P[r + 3] * b1 + P[r + 6] * b2) * w;
      }
      double2* go = reinterpret_cast<double2*>(I.Gloc + 12 * (size_t)e);
#pragma unroll
      for (int k = 0; k < 6; ++k) go[k] = make_double2(g[2 * k], g[2 * k + 1]);
      I.Eloc[e] = Ee;
    }
    double p[1] = {Ee}, tot[1];
    if (tile_done<1>(I, lt, tiles_of(I.m), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_ELEM_EG);
      st->E_el = tot[0];
    }
  }
}

// Element energies of the line-search trials evaluated together (PH_EVALK): for each
// trial k, x = xs + a_k dx is formed node by node exactly as the vector-op stage forms a
// trial point, and the element energy exactly as st_elem_eg does, so each trial's total
// has the bits a one-at-a-time evaluation would give.  Energies only (the accepted trial
// is evaluated again with its gradient).
__device__ __forceinline__ void st_elem_ek(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_EVALK) continue;
    const int K = st->lsk;
    const int e = lt * kTile + threadIdx.x;
    double Ek[kLsK];
#pragma unroll
    for (int k = 0; k < kLsK; ++k) Ek[k] = 0.0;
    if (e < I.m) {
      const int4 tt = reinterpret_cast<const int4*>(I.tets)[e];
      const int nd[4] = {tt.x, tt.y, tt.z, tt.w};
      double xs[4][3], dx[4][3], X[4][3];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        ld4(I.xs, nd[a], xs[a]);
        ld4(I.dx, nd[a], dx[a]);
        ld4(I.xrest, nd[a], X[a]);
      }
      double R[12];
      const double2* r2 = reinterpret_cast<const double2*>(I.rest64 + 12 * (size_t)e);
#pragma unroll
      for (int k = 0; k < 6; ++k) { double2 q = r2[k]; R[2 * k] = q.x; R[2 * k + 1] = q.y; }
      const double w = R[9], lam = R[10], mu = R[11];
      const int model = I.model[e];
      for (int k = 0; k < K; ++k) {
        const double ak = st->ls_a[k];
        double x[4][3];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) x[a][c] = xs[a][c] + ak * dx[a][c];
        double u0[3], Du[9];
#pragma unroll
        for (int r = 0; r < 3; ++r) u0[r] = x[0][r] - X[0][r];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < 3; ++r) Du[r + 3 * c] = (x[c + 1][r] - X[c + 1][r]) - u0[r];
        double Hd[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < 3; ++r)
            Hd[r + 3 * c] = Du[r] * R[0 + 3 * c] + Du[r + 3] * R[1 + 3 * c] + Du[r + 6] * R[2 + 3 * c];
        double psi, P[9];
        bool inverted;
        material_eg(model, lam, mu, Hd, &psi, P, &inverted);
        Ek[k] = inverted ? __longlong_as_double(0x7ff0000000000000LL) : psi * w;
      }
    }
    double tot[kLsK];
    if (tile_done<kLsK>(I, lt, tiles_of(I.m), ncta, Ek, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_ELEM_EG);
      for (int k = 0; k < K; ++k) st->ls_eel[k] = tot[k];
      st->phase = PH_EVALK2;
      advance(B, i);
    }
  }
}

// Linear-load (and inertia) energies of the trials, formed per node exactly as st_gather
// forms them; then the trials' totals go to the line-search scan.
__device__ __forceinline__ void st_lin_ek(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_EVALK2) continue;
    const int K = st->lsk;
    const int v = lt * kTile + threadIdx.x;
    double Lk[kLsK];
#pragma unroll
    for (int k = 0; k < kLsK; ++k) Lk[k] = 0.0;
    if (v < I.n) {
      double xs[3], dx[3], h[3];
      ld4(I.xs, v, xs);
      ld4(I.dx, v, dx);
      ld4(I.hlin, v, h);
      const bool dyn = I.opts->dynamic != 0;
      double x0[3] = {0.0, 0.0, 0.0}, v0[3] = {0.0, 0.0, 0.0};
      const double dt = I.opts->dt, m = dyn ? I.mass[v] : 0.0;
      if (dyn) {
        ld4(I.x0, v, x0);
        ld4(I.v0, v, v0);
      }
      const SoftNode sk = ld_soft(I, v);
      for (int k = 0; k < K; ++k) {
        const double ak = st->ls_a[k];
        double x[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = xs[c] + ak * dx[c];
        double elin = x[0] * h[0] + x[1] * h[1] + x[2] * h[2];
        if (dyn) {
          double acc = 0.0;
          for (int c = 0; c < 3; ++c) {
            double a = (x[c] - x0[c]) / (dt * dt) - v0[c] / dt;
            acc += a * (m * a);
          }
          elin += (dt * dt / 2.0) * acc;
        }
        if (sk.k != 0.0) elin += soft_energy(sk, x, nullptr);
        Lk[k] = elin;
      }
    }
    double tot[kLsK];
    if (tile_done<kLsK>(I, lt, tiles_of(I.n), ncta, Lk, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_GATHER);
      for (int k = 0; k < K; ++k) st->ls_e[k] = st->ls_eel[k] + tot[k];
      st->phase = PH_EVAL_DONE;  // purpose 2: the scan of ctl_lsk_check
      advance(B, i);
    }
  }
}

__global__ void __launch_bounds__(kTile) k_elem_eg(BatchDev B) {
  extern __shared__ __align__(16) unsigned char smraw[];  // staged nodes of the served path
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_elem_eg(B, full_map(B, B.pre_tet), blockIdx.x, gridDim.x, sm, flag, smraw);
}

// node gather of element gradients + linear loads (+ inertia), energy and ||g||^2
__device__ __forceinline__ void st_gather(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_EVAL) continue;
    const int v = lt * kTile + threadIdx.x;
    double p[3] = {0.0, 0.0, 0.0};
    if (v < I.n) {
      double g[3] = {0.0, 0.0, 0.0};
      const int c0 = I.nseg_ptr[v], c1 = I.nseg_ptr[v + 1];
      int c = c0;
      // four contributions in flight (ids, then values), added in element order
      for (; c + 4 <= c1; c += 4) {
        int id[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) id[u] = I.nseg_c[c + u];
        double val[4][3];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const double* src = I.Gloc + 3 * (size_t)id[u];
          val[u][0] = src[0]; val[u][1] = src[1]; val[u][2] = src[2];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) { g[0] += val[u][0]; g[1] += val[u][1]; g[2] += val[u][2]; }
      }
      for (; c < c1; ++c) {
        const double* src = I.Gloc + 3 * (size_t)I.nseg_c[c];
        g[0] += src[0]; g[1] += src[1]; g[2] += src[2];
      }
      double h[3], x[3];
      ld4(I.hlin, v, h);
      ld4(I.x, v, x);
      double elin = x[0] * h[0] + x[1] * h[1] + x[2] * h[2];
      for (int c = 0; c < 3; ++c) g[c] += h[c];
      if (I.opts->dynamic) {
        const double dt = I.opts->dt, m = I.mass[v];
        double x0[3], v0[3], acc = 0.0;
        ld4(I.x0, v, x0);
        ld4(I.v0, v, v0);
        for (int c = 0; c < 3; ++c) {
          double a = (x[c] - x0[c]) / (dt * dt) - v0[c] / dt;
          g[c] += m * a;
          acc += a * (m * a);
        }
        elin += (dt * dt / 2.0) * acc;
      }
      const SoftNode sk = ld_soft(I, v);
      if (sk.k != 0.0) elin += soft_energy(sk, x, g);
      if (!st->nofix) {
        const int fm = I.fixmask[v];
        for (int c = 0; c < 3; ++c)
          if (fm & (1 << c)) g[c] = 0.0;
      }
      st4(I.gn, v, g);
      p[0] = elin;
      p[1] = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
      if (I.opts->lsearch_type >= 3) {  // dx . g of the trial, for the Wolfe line searches
        double d[3];
        ld4(I.dx, v, d);
        p[2] = d[0] * g[0] + d[1] * g[1] + d[2] * g[2];
      }
    }
    double tot[3];
    if (tile_done<3>(I, lt, tiles_of(I.n), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_GATHER);
      st->E_eval = st->E_el + tot[0];
      st->gg_eval = tot[1];
      st->dg_eval = tot[2];
      st->phase = PH_EVAL_DONE;
      advance(B, i);
    }
  }
}

__global__ void __launch_bounds__(kTile) k_gather(BatchDev B) {
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_gather(B, full_map(B, B.pre_node), blockIdx.x, gridDim.x, sm, flag);
}

// ---------------------------------------------------------------------------
// element Hessian: the 10 node blocks of H_e = w DFDx^T dP/dF DFDx in closed form.
// With B_a the shape-function gradients and u_a a per-node 3-vector,
//   H_np = w [ s_np I + lam u_n u_p^T + beta u_p u_n^T + t_np M ]
//   CoNH: u_a = F^-T B_a, s = mu B_n.B_p, beta = mu - lam/2 log J^2, t = 0
//   StVK: u_a = F B_a,    s = B_n^T S B_p, beta = mu, t = mu B_n.B_p, M = F F^T
// Each block is written oriented as the global lower block (row node = larger id).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void elem_blocks(const InstDev& I, int e, Real* out /* 90, stride 1 */) {
  int nd[4];
  double Du[9];
  load_du(I, e, nd, Du);
  elem_blocks_core<Real>(nd, Du, I.rest64 + 12 * (size_t)e, PcgBufs<Real>::rest(I) + 12 * (size_t)e, I.model[e], out);
}

template <typename Real>
__device__ __forceinline__ void st_elem_hess(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag, unsigned char* smraw) {
  Real* sh = reinterpret_cast<Real*>(smraw);  // [kTile][90]
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    if (I.st->phase != PH_HESS) continue;
    const int e0 = lt * kTile;
    const int cnt = min(kTile, I.m - e0);
    if ((int)threadIdx.x < cnt) elem_blocks<Real>(I, e0 + threadIdx.x, sh + threadIdx.x * 90);
    __syncthreads();
    Real* dst = PcgBufs<Real>::Hloc(I) + (size_t)e0 * 90;
    for (int k = threadIdx.x; k < cnt * 90; k += blockDim.x) dst[k] = sh[k];
    __syncthreads();
  }
}

template <typename Real>
__global__ void __launch_bounds__(kTile) k_elem_hess(BatchDev B) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_elem_hess<Real>(B, full_map(B, B.pre_tet), blockIdx.x, gridDim.x, sm, flag, smraw);
}

// ---------------------------------------------------------------------------
// assembly: one 9-lane group per lower block sums its contributions in element
// order (the segment list), applies inertia and FixMatrixDoFs, and writes the
// block and its transpose into the SELL matrix; ||A||_F^2 of the stored lower
// entries is reduced for the regularisation threshold (LinearSolver.cpp:57-66).
// ---------------------------------------------------------------------------
template <typename Real>
__device__ __forceinline__ void st_assemble(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_HESS) continue;
    const Real* Hloc = PcgBufs<Real>::Hloc(I);
    Real* H = PcgBufs<Real>::H(I);
    const bool dyn = I.opts->dynamic != 0, nofix = st->nofix != 0;
    const double dt = I.opts->dt;
    Real nrm = 0;  // ||A||_F^2 of the stored entries, for the regularisation threshold only
    // one thread per stored block, its nine entries together: the contributions' ids four at
    // a time, then their nine values each, so that a block costs few dependent round trips;
    // every entry adds its contributions in element order
    const int k = lt * kTile + threadIdx.x;
    if (k < I.nlo) {
      Real s[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) s[e] = 0;
      const int c0 = I.seg_ptr[k], c1 = I.seg_ptr[k + 1];
      int c = c0;
      for (; c + 4 <= c1; c += 4) {
        int id[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) id[u] = I.seg_c[c + u];
        Real val[4][9];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int e = 0; e < 9; ++e) val[u][e] = Hloc[(size_t)id[u] * 9 + e];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int e = 0; e < 9; ++e) s[e] += val[u][e];
      }
      for (; c < c1; ++c) {
        const Real* hv = Hloc + (size_t)I.seg_c[c] * 9;
#pragma unroll
        for (int e = 0; e < 9; ++e) s[e] += hv[e];
      }
      const int R = I.lo_rc[2 * k], C = I.lo_rc[2 * k + 1];
      const int64_t lo = I.lo_slot[k], up = R != C ? I.up_slot[k] : -1;
      Real* const Hlo = H + sell_addr(lo, 0);  // entry e of a slot at +32 e
      Real* const Hup = up >= 0 ? H + sell_addr(up, 0) : nullptr;
      const int fr = nofix ? 0 : I.fixmask[R], fc = nofix ? 0 : I.fixmask[C];
      // diagonal blocks: + M/dt^2 of the dynamic problem, + k I of a soft fixed position
      const double ks = (I.soft && R == C) ? I.soft[4 * (size_t)R + 3] : 0.0;
      const bool diag = (dyn && R == C) || ks != 0.0;
      const Real md = diag ? (Real)((dyn ? I.mass[R] / (dt * dt) : 0.0) + ks) : (Real)0;
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        const int a = e / 3, b = e % 3;
        Real v = s[e];
        if (diag && a == b) v += md;
        if (((fr >> a) | (fc >> b)) & 1) v = (R == C && a == b) ? (Real)1 : (Real)0;
        Hlo[32 * e] = v;
        if (Hup) Hup[32 * (b * 3 + a)] = v;
        nrm += v * v;
      }
    }
    Real p[1] = {nrm};
    double tot[1];
    if (tile_done<1>(I, lt, tiles_of(I.nlo), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_ELEM_HESS);  // the element kernel ran on this instance in the same round
      count_bytes(B, I, K_ASSEMBLE);
      st->normA2 = tot[0];
      st->regT = 1e-6 * sqrt(tot[0]);
    }
  }
}

template <typename Real>
__global__ void __launch_bounds__(kTile) k_assemble(BatchDev B) {
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_assemble<Real>(B, full_map(B, B.pre_lob), blockIdx.x, gridDim.x, sm, flag);
}

// preconditioner: inverse of each node's 3x3 diagonal block (+ shift), or of its diagonal
template <typename Real>
__device__ __forceinline__ void st_jacobi(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_HESS && st->phase != PH_JACOBI) continue;
    const int v = lt * kTile + threadIdx.x;
    if (v < I.n) {
      const Real* H = PcgBufs<Real>::H(I);
      Real* Mi = PcgBufs<Real>::minv(I);
      const int64_t s = I.diag_slot[v];
      double D[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) D[k] = (double)H[sell_addr(s, k)];  // row-major a*3+b
      D[0] += st->shift; D[4] += st->shift; D[8] += st->shift;
      double inv[9];
      if (I.opts->precond == 1) {
        double C[9];
        cof3(D, C);  // symmetric: cofactor == adjugate^T == adjugate
        double d = D[0] * C[0] + D[3] * C[3] + D[6] * C[6];
        if (d != 0.0 && isfinite(d)) {
#pragma unroll
          for (int k = 0; k < 9; ++k) inv[k] = C[k] / d;
        } else {
#pragma unroll
          for (int k = 0; k < 9; ++k) inv[k] = (k % 4 == 0) ? 1.0 : 0.0;
        }
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) inv[k] = 0.0;
        inv[0] = D[0] != 0.0 ? 1.0 / D[0] : 1.0;
        inv[4] = D[4] != 0.0 ? 1.0 / D[4] : 1.0;
        inv[8] = D[8] != 0.0 ? 1.0 / D[8] : 1.0;
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) Mi[(size_t)k * I.n + v] = (Real)inv[k];
    }
    if (tile_count_done(I, lt, tiles_of(I.n), ncta, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_JACOBI);
      st->phase = PH_LINSETUP;
      advance(B, i);
    }
  }
}

// b = -g, dx = guess (previous accepted step, EigenCG solveWithGuess) or 0
__device__ __forceinline__ void st_linsetup(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_LINSETUP) continue;
    const int v = lt * kTile + threadIdx.x;
    double p[1] = {0.0};
    if (v < I.n) {
      double g[3], d[3] = {0.0, 0.0, 0.0};
      ld4(I.g, v, g);
      for (int c = 0; c < 3; ++c) g[c] = -g[c];
      st4(I.bvec, v, g);
      if (I.opts->warm_guess) ld4(I.dxprev, v, d);
      if (I.opts->precision != 0 && !st->nofix) {
        // the served path's inexact FP32 solves start the fixed DoFs at their exact step, 0:
        // their rows and columns are the identity and their right-hand side is 0, so the PCG
        // keeps them at 0 and a clamp never drifts by the inner tolerance times a guess (a
        // staged clamp's move enters the guess as x - x_prev does in the reference)
        const int fm = I.fixmask[v];
        for (int c = 0; c < 3; ++c)
          if (fm & (1 << c)) d[c] = 0.0;
      }
      st4(I.dx, v, d);
      p[0] = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    }
    double tot[1];
    if (tile_done<1>(I, lt, tiles_of(I.n), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_LINSETUP);
      const double tol = st->lin_tol;
      st->bb = tot[0];
      st->thr_final = fmax(tol * tol * tot[0], DBL_MIN);
      st->sweeps = 0;
      st->lin_status = LIN_RUNNING;
      if (tot[0] == 0.0) {  // zero right-hand side: x = 0
        st->lin_status = LIN_CONVERGED;
        st->b_dot_dx = 0.0;
        st->dx_norm = 0.0;
        st->vecop = VO_ZERODX;
        st->next_phase = PH_LIN_DONE;
        st->phase = PH_VEC;
      } else {
        st->phase = PH_RESID;
      }
      advance(B, i);
    }
  }
}


// SELL-32 row sweep: acc = sum_k H(row, col_k) * X(col_k), X given per column by a functor.
// Slots are taken 4 at a time: all column ids, then all gathers and block loads are issued
// before the arithmetic, so one row costs a few memory round trips instead of one per slot
// (what bounds the sweep when only a few small instances are still iterating).
template <typename Real, typename Acc, typename GetX>
__device__ __forceinline__ void sell_row(const InstDev& I, const Real* H, int v, GetX getx, Acc (&acc)[3]) {
  const int c = v >> 5, lane = v & 31;
  const int s0 = __ldg(I.chunk_off + c);
  const int len = (__ldg(I.chunk_off + c + 1) - s0) >> 5;
  acc[0] = acc[1] = acc[2] = (Acc)0;
  for (int k0 = 0; k0 < len; k0 += 4) {
    int col[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) col[u] = (k0 + u < len) ? __ldg(I.slot_col + (int64_t)s0 + (k0 + u) * 32 + lane) : v;
    Acc xc[4][3];
#pragma unroll
    for (int u = 0; u < 4; ++u) getx(col[u], xc[u]);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (k0 + u < len) {
        const int64_t s = (int64_t)s0 + (k0 + u) * 32 + lane;
        const Real* hp = H + (s >> 5) * 288 + (s & 31);
        Acc h[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) h[q] = (Acc)hp[q * 32];
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a] += h[3 * a] * xc[u][0] + h[3 * a + 1] * xc[u][1] + h[3 * a + 2] * xc[u][2];
      }
    }
  }
}

// L lanes per row (L = 1, 2 or 4; lanes L*r .. L*r+L-1 of the calling warp share row v):
// lane `sub` takes slots sub, sub+L, ..., four at a time -- their column ids and blocks
// are loaded together, then the four gathers, then the arithmetic -- so four slots cost
// two dependent memory round trips; the partial sums are combined with xor-shuffles and
// every lane of the group ends with the full row.
template <int L, typename Real, typename Acc, typename GetX>
__device__ __forceinline__ void sell_row_lanes(const InstDev& I, const Real* H, int v, int sub, bool valid, GetX getx,
                                               Acc (&acc)[3]) {
  acc[0] = acc[1] = acc[2] = (Acc)0;
  if (valid) {
    const int c = v >> 5, lane = v & 31;
    const int s0 = __ldg(I.chunk_off + c);
    const int len = (__ldg(I.chunk_off + c + 1) - s0) >> 5;
    for (int k0 = sub; k0 < len; k0 += 4 * L) {
      int col[4];
      Acc h[4][9];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + u * L;
        const bool in = k < len;
        const int64_t s = (int64_t)s0 + (int64_t)(in ? k : 0) * 32 + lane;
        col[u] = in ? __ldg(I.slot_col + s) : -1;
        const Real* hp = H + (s >> 5) * 288 + (s & 31);
#pragma unroll
        for (int q = 0; q < 9; ++q) h[u][q] = in ? (Acc)hp[q * 32] : (Acc)0;
      }
      Acc xc[4][3];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (col[u] >= 0) {
          getx(col[u], xc[u]);
        } else {
          xc[u][0] = xc[u][1] = xc[u][2] = (Acc)0;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int a = 0; a < 3; ++a) acc[a] += h[u][3 * a] * xc[u][0] + h[u][3 * a + 1] * xc[u][1] + h[u][3 * a + 2] * xc[u][2];
    }
  }
#pragma unroll
  for (int off = 1; off < L; off <<= 1)
#pragma unroll
    for (int a = 0; a < 3; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], off);
}

template <typename Real, typename Acc, typename GetX>
__device__ __forceinline__ void sell_row_quad(const InstDev& I, const Real* H, int v, int sub, bool valid, GetX getx,
                                              Acc (&acc)[3]) {
  sell_row_lanes<4, Real, Acc>(I, H, v, sub, valid, getx, acc);
}

// r64 = b - (H + shift I) dx in FP64 (FP32 values promoted); starts an inner PCG on r
template <typename Real>
__device__ __forceinline__ void st_resid(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_RESID) continue;
    const int v = lt * kTile + threadIdx.x;
    double p[5] = {0, 0, 0, 0, 0};
    if (v < I.n) {
      const Real* H = PcgBufs<Real>::H(I);
      double acc[3];
      const double* dxv = I.dx;
      sell_row<Real, double>(I, H, v, [&](int col, double (&xc)[3]) { ld4(dxv, col, xc); }, acc);
      double xv[3], b[3];
      ld4(I.dx, v, xv);
      ld4(I.bvec, v, b);
      const double sh = st->shift;
      double r[3];
      for (int a = 0; a < 3; ++a) r[a] = b[a] - (acc[a] + sh * xv[a]);
      st4(I.r64, v, r);
      p[0] = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      p[1] = b[0] * xv[0] + b[1] * xv[1] + b[2] * xv[2];
      p[2] = xv[0] * xv[0] + xv[1] * xv[1] + xv[2] * xv[2];
      // inner PCG start: e = 0, r = (Real) r64, z = Minv r, p_prev = 0
      Real rr_[3] = {(Real)r[0], (Real)r[1], (Real)r[2]}, zero[3] = {0, 0, 0}, z[3];
      const Real* Mi = PcgBufs<Real>::minv(I);
      for (int a = 0; a < 3; ++a)
        z[a] = Mi[(size_t)(3 * a) * I.n + v] * rr_[0] + Mi[(size_t)(3 * a + 1) * I.n + v] * rr_[1] +
               Mi[(size_t)(3 * a + 2) * I.n + v] * rr_[2];
      st4(PcgBufs<Real>::r(I), v, rr_);
      st4(PcgBufs<Real>::z(I), v, z);
      st4(PcgBufs<Real>::e(I), v, zero);
      st4(PcgBufs<Real>::pa(I), v, zero);
      p[3] = (double)(rr_[0] * z[0] + rr_[1] * z[1] + rr_[2] * z[2]);
      p[4] = (double)(rr_[0] * rr_[0] + rr_[1] * rr_[1] + rr_[2] * rr_[2]);
    }
    double tot[5];
    if (tile_done<5>(I, lt, tiles_of(I.n), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_RESID);
      st->rr64 = tot[0];
      st->b_dot_dx = tot[1];
      st->dx_norm = sqrt(tot[2]);
      const bool conv = tot[0] < st->thr_final;
      if (conv || st->sweeps >= I.opts->max_refine_sweeps || st->lin_status == LIN_TRUNCATED) {
        if (st->lin_status == LIN_TRUNCATED) {
        } else if (conv) st->lin_status = LIN_CONVERGED;
        else if (st->lin_status == LIN_RUNNING) st->lin_status = LIN_MAXITER;
        st->phase = PH_LIN_DONE;
      } else {
        const double it = I.opts->inner_tol;
        st->thr_inner = (I.opts->precision == 0) ? st->thr_final : fmax(it * it * tot[0], st->thr_final);
        st->rz = tot[3];
        st->rr = tot[4];
        st->pcg_iter = 0;
        st->pcg_parity = 0;
        st->beta = 0.0;
        st->truncate = 0;
        st->pcg_resume = 0;
        st->lin_status = LIN_RUNNING;
        st->phase = PH_PCG;
      }
      advance(B, i);
    }
  }
}


// PCG step 1: p = z + beta p_prev (formed on the fly for every column, written
// for the own row into the other buffer), q = (H + shift I) p, pq = p.q
// kGrid: run by k_gpcg_a (the whole-GPU PCG kernel, instances of PCG kind 3) instead of the
// engine (instances not left to a cluster or grid kernel); the iteration is the same.
template <typename Real, bool kGrid = false>
__device__ __forceinline__ bool pcg_here(const BatchDev& B, const InstDev& I) {
  return kGrid ? I.pcg_cluster == 3 : !cluster_owned(B, I);
}
// an instance of PCG kind 3 leaves the grid kernel's loop
__device__ __forceinline__ void gpcg_left(int32_t* left) {
  if (left) atomicSub(left, 1);
}
// advance() out of line, for the small kernels: its state copy stays off their registers
__device__ __noinline__ void advance_ool(const BatchDev& B, int i) { advance(B, i); }
template <bool kGrid>
__device__ __forceinline__ void advance_pcg(const BatchDev& B, int i) {
  if (kGrid) advance_ool(B, i);
  else advance(B, i);
}

template <typename Real, bool kGrid = false>
__device__ __forceinline__ void st_pcg_a(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag,
                                         int32_t* left = nullptr) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    std::conditional_t<kGrid, const InstDev&, const InstDev> I = B.inst[i];  // the engine keeps a copy in registers
    NState* st = I.st;
    if (st->phase != PH_PCG || !pcg_here<Real, kGrid>(B, I)) continue;
    Real p[1] = {(Real)0};  // per-tile inner product in the PCG's own precision
    {
      const int par = st->pcg_parity;
      const Real* pold = par ? PcgBufs<Real>::pb(I) : PcgBufs<Real>::pa(I);
      Real* pnew = par ? PcgBufs<Real>::pa(I) : PcgBufs<Real>::pb(I);
      const Real* z = PcgBufs<Real>::z(I);
      const Real beta = (Real)st->beta, sh = (Real)st->shift;
      auto getx = [&](int col, Real (&xc)[3]) {
        Real zc[3], pc[3];
        ld4(z, col, zc);
        ld4(pold, col, pc);
        for (int a = 0; a < 3; ++a) xc[a] = zc[a] + beta * pc[a];
      };
      // one-chunk tiles: 32 rows x 4 lanes; four-chunk tiles: one row per thread, so that a
      // warp's load of a block plane is one 128-byte line of the slot-row (the wide form
      // spreads it over four lines, and the whole-GPU SpMV is bound by L2 requests)
      const bool wide = pcg_cpt(I) == 1;
      const int sub = wide ? (threadIdx.x & 3) : 0, row = wide ? (threadIdx.x >> 2) : threadIdx.x;
      const int ch0 = wide ? lt : 4 * lt, ch1 = wide ? ch0 + 1 : min(ch0 + 4, I.nchunks);
      for (int ch = ch0; ch < ch1; ch += wide ? 1 : 4) {
        const int v = ch * 32 + row;
        const bool valid = v < I.n;
        Real acc[3];
        if (wide) sell_row_quad<Real, Real>(I, PcgBufs<Real>::H(I), v, sub, valid, getx, acc);
        else sell_row_lanes<1, Real, Real>(I, PcgBufs<Real>::H(I), v, 0, valid, getx, acc);
        if (valid && sub == 0) {
          Real zv[3], pv[3];
          ld4(z, v, zv);
          ld4(pold, v, pv);
          for (int a = 0; a < 3; ++a) {
            pv[a] = zv[a] + beta * pv[a];
            acc[a] += sh * pv[a];
          }
          st4(pnew, v, pv);
          st4(PcgBufs<Real>::q(I), v, acc);
          p[0] += pv[0] * acc[0] + pv[1] * acc[1] + pv[2] * acc[2];
        }
      }
    }
    double tot[1];
    if (tile_done<1>(I, lt, pcg_tiles(B, I), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_PCG_A);
      st->pq = tot[0];
      if ((I.opts->precision == 0 || I.opts->curv_through) && tot[0] < 0.0) {
        // Eigen's ConjugateGradient has no curvature test: a negative p.q gives a negative
        // step along p and the iteration goes on; LinearSolver_EigenCG regularises only
        // when the result fails b.x >= 0 (LinearSolver_EigenCG.cpp:95-107)
        st->alpha = st->rz / tot[0];
      } else if (!(tot[0] > 0.0)) {  // not positive definite along p (or non-finite)
        if (I.opts->precision != 0 && tot[0] < 0.0 && st->pcg_iter == 0) {
          // truncated CG, first direction: step along p with |p.q| and stop
          st->alpha = st->rz / -tot[0];
          st->truncate = 1;
        } else {
          st->lin_status = (I.opts->precision != 0 && tot[0] < 0.0) ? LIN_TRUNCATED : LIN_BREAKDOWN;
          st->phase = (st->lin_status == LIN_TRUNCATED) ? PH_ACCUM : PH_LIN_DONE;
          advance_pcg<kGrid>(B, i);
          if (kGrid) gpcg_left(left);
        }
      } else {
        st->alpha = st->rz / tot[0];
      }
    }
  }
}


// PCG step 2: e += alpha p, r -= alpha q, z = Minv r; convergence ||r||^2 < thr (Eigen's rule)
template <typename Real, bool kGrid = false>
__device__ __forceinline__ void st_pcg_b(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag,
                                         int32_t* left = nullptr) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    std::conditional_t<kGrid, const InstDev&, const InstDev> I = B.inst[i];  // the engine keeps a copy in registers
    NState* st = I.st;
    if (st->phase != PH_PCG || !pcg_here<Real, kGrid>(B, I)) continue;
    const int cpt = pcg_cpt(I);
    const int v = lt * cpt * 32 + threadIdx.x;  // one row per thread over the tile's chunks
    Real p[2] = {(Real)0, (Real)0};  // per-tile inner products in the PCG's own precision
    if ((int)threadIdx.x < cpt * 32 && v < I.n) {
      const Real alpha = (Real)st->alpha;
      const Real* pc = st->pcg_parity ? PcgBufs<Real>::pa(I) : PcgBufs<Real>::pb(I);
      Real pv[3], qv[3], ev[3], rv[3], z[3];
      ld4(pc, v, pv);
      ld4(PcgBufs<Real>::q(I), v, qv);
      ld4(PcgBufs<Real>::e(I), v, ev);
      ld4(PcgBufs<Real>::r(I), v, rv);
      for (int a = 0; a < 3; ++a) {
        ev[a] += alpha * pv[a];
        rv[a] -= alpha * qv[a];
      }
      const Real* Mi = PcgBufs<Real>::minv(I);
      for (int a = 0; a < 3; ++a)
        z[a] = Mi[(size_t)(3 * a) * I.n + v] * rv[0] + Mi[(size_t)(3 * a + 1) * I.n + v] * rv[1] +
               Mi[(size_t)(3 * a + 2) * I.n + v] * rv[2];
      st4(PcgBufs<Real>::e(I), v, ev);
      st4(PcgBufs<Real>::r(I), v, rv);
      st4(PcgBufs<Real>::z(I), v, z);
      p[0] = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
      p[1] = rv[0] * z[0] + rv[1] * z[1] + rv[2] * z[2];
    }
    double tot[2];
    if (tile_done<2>(I, lt, pcg_tiles(B, I), ncta, p, tot, sm, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_PCG_B);
      st->pcg_iter++;
      st->pcg_total++;
      st->rr = tot[0];
      if (st->truncate) {
        st->truncate = 0;
        st->lin_status = LIN_TRUNCATED;
        st->phase = PH_ACCUM;
      } else if (tot[0] < st->thr_inner) {
        st->lin_status = LIN_CONVERGED;
        st->phase = PH_ACCUM;
      } else if (st->pcg_iter >= I.opts->ls_num_max_iters) {
        st->lin_status = LIN_MAXITER;
        st->phase = PH_ACCUM;
      } else {
        st->beta = tot[1] / st->rz;
        st->rz = tot[1];
        st->pcg_parity ^= 1;
      }
      if (st->phase != PH_PCG) {
        advance_pcg<kGrid>(B, i);
        if (kGrid) gpcg_left(left);
      }
    }
  }
}


// dx += e (FP64), then back to the FP64 residual
template <typename Real>
__device__ __forceinline__ void st_accum(const BatchDev& B, const TileMap& M, int cta, int ncta, double* sm, int& flag) {
  const int total = map_total(M);
  for (int t = cta; t < total; t += ncta) {
    int i, lt;
    map_tile(M, t, i, lt);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (st->phase != PH_ACCUM) continue;
    const int v = lt * kTile + threadIdx.x;
    if (v < I.n) {
      Real ev[3];
      double d[3];
      ld4(PcgBufs<Real>::e(I), v, ev);
      ld4(I.dx, v, d);
      for (int a = 0; a < 3; ++a) d[a] += (double)ev[a];
      st4(I.dx, v, d);
    }
    if (tile_count_done(I, lt, tiles_of(I.n), ncta, &flag) && threadIdx.x == 0) {
      count_bytes(B, I, K_ACCUM);
      st->sweeps++;
      st->total_sweeps++;
      st->phase = PH_RESID;
      advance(B, i);
    }
  }
}


// ---------------------------------------------------------------------------
// the persistent engine: whole Newton rounds in one cooperative launch
// ---------------------------------------------------------------------------
// Grid barrier over all CTAs of a cooperative launch (co-residency is guaranteed by
// cudaLaunchCooperativeKernel).  The wait is bounded: after `limit` clock cycles
// (kBarrierLimit by default) a CTA records a timeout and the stage it was in, and every
// CTA then leaves the kernel at its next barrier, so a fault in the engine ends the
// launch instead of hanging the device.  The barrier touches global memory only.

// nblocks = the CTAs taking part (always the lowest-numbered ones).
// `abort` is the launch-wide error flag (the round-wide barrier's): a timeout on either
// barrier object raises it and every waiting CTA leaves.
// live: the per-phase counts; the last CTA to arrive copies them into the snapshot half
// that every CTA reads after the barrier (null: no counts).
// unmet: the barrier expects one arrival more than nblocks, which never comes (the test
// hook of phx_debug_unmet_barrier): every CTA waits until the limit.
__device__ __forceinline__ bool grid_sync(GridBar* gb, unsigned int nblocks, int tag, int* abort,
                                          int32_t* live = nullptr, long long limit = kBarrierLimit,
                                          bool unmet = false) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &gb->gen;
    volatile int* verr = abort;
    const unsigned int g = *vgen;
    __threadfence();
    const unsigned int a = atomicAdd(&gb->arrive, 1u);
    if (!unmet && a == nblocks - 1) {
      gb->arrive = 0u;
      if (live) {
        __threadfence();
        for (int k = 0; k < 16; ++k) live[16 + k] = *(volatile int32_t*)(live + k);
      }
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      const long long t0 = clock64();
      int polls = 0;
      while (*vgen == g) {
        if (*verr) break;
        if (clock64() - t0 > limit) {
          if (atomicCAS(&gb->err, 0, 1) == 0) gb->stage = tag;
          atomicExch(abort, 1);
          break;
        }
        if (++polls > 64) __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)abort == 0;
}

// block-wide exclusive scan of 4 ints; returns totals in tot (all threads)
__device__ __forceinline__ void block_scan4(int (&v)[4], int (&tot)[4], int* sm /* [32*4] */) {
  // (four running sums at once; compact() runs two of these passes)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int inc[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    inc[k] = v[k];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, inc[k], off);
      if (lane >= off) inc[k] += y;
    }
  }
  __syncthreads();
  if (lane == 31)
#pragma unroll
    for (int k = 0; k < 4; ++k) sm[warp * 4 + k] = inc[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int w = lane < nw ? sm[lane * 4 + k] : 0;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, off);
        if (lane >= off) w += y;
      }
      if (lane < nw) sm[lane * 4 + k] = w;  // inclusive warp prefix
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int before = warp > 0 ? sm[(warp - 1) * 4 + k] : 0;
    tot[k] = sm[(nw - 1) * 4 + k];
    v[k] = before + inc[k] - v[k];  // exclusive
  }
  __syncthreads();
}

// One CTA: starts new solves, publishes phases, and lists the instances not yet done
// with the prefix of their tet, node and lower-block tile counts.  It also sizes the
// round: act[1] = CTAs that take part (no more than the CTAs still running, act[1] of
// the previous round), act[2] = CTAs that take part in the PCG block.
__device__ void compact(const BatchDev& B, const EngineArgs& A) {
  __shared__ int scan_sm[32 * 4];
  const int num = *B.num;
  for (int i = threadIdx.x; i < num; i += blockDim.x) {
    const int ph = *(volatile int32_t*)&B.inst[i].st->phase;
    if (ph == PH_START) advance(B, i);
    else B.flags[8 + i] = ph;
  }
  __syncthreads();
  __shared__ int cnt[16];
  if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < num; i += blockDim.x) {
    const int ph = B.flags[8 + i];
    if (ph > PH_DONE && ph < kBucketClusterPcg) atomicAdd(&cnt[phase_bucket(B, B.inst[i], ph)], 1);
  }
  __syncthreads();
  if (B.phase_live && threadIdx.x < 16) {
    B.phase_live[threadIdx.x] = cnt[threadIdx.x];
    B.phase_live[16 + threadIdx.x] = cnt[threadIdx.x];
  }
  int* ids = A.act + 4;
  int* pt = ids + A.cap;
  int* pn = pt + A.cap + 1;
  int* pl = pn + A.cap + 1;
  int* pp = pl + A.cap + 1;
  int run[4] = {0, 0, 0, 0};
  int run_pcg = 0;
  __shared__ int eng_pcg_tiles, cluster_waiting;
  if (threadIdx.x == 0) {
    eng_pcg_tiles = 0;
    cluster_waiting = 0;
  }
  __syncthreads();
  for (int base = 0; base < num; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const bool act = i < num && B.flags[8 + i] != PH_DONE;
    const int ptiles = act ? pcg_tiles(B, B.inst[i]) : 0;
    if (act && !cluster_owned(B, B.inst[i])) atomicAdd(&eng_pcg_tiles, ptiles);
    if (act && cluster_owned(B, B.inst[i]) && B.flags[8 + i] == PH_PCG) atomicAdd(&cluster_waiting, 1);
    int c[4] = {act ? 1 : 0, act ? tiles_of(B.inst[i].m) : 0, act ? tiles_of(B.inst[i].n) : 0,
                act ? tiles_of(B.inst[i].nlo) : 0};
    int ex[4] = {c[0], c[1], c[2], c[3]}, tot[4];
    block_scan4(ex, tot, scan_sm);
    int e2[4] = {ptiles, 0, 0, 0}, t2[4];
    block_scan4(e2, t2, scan_sm);
    if (act) {
      const int pos = run[0] + ex[0];
      ids[pos] = i;
      pt[pos + 1] = run[1] + ex[1] + c[1];
      pn[pos + 1] = run[2] + ex[2] + c[2];
      pl[pos + 1] = run[3] + ex[3] + c[3];
      pp[pos + 1] = run_pcg + e2[0] + ptiles;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) run[k] += tot[k];
    run_pcg += t2[0];
  }
  if (A.wait) {
    // the instances waiting for each PCG kind, in corder's order (largest first), the kind-3
    // PCG tile prefix, and the counters reset: the cluster and grid PCG kernels launched next
    // work through these lists
    int32_t* W = A.wait;
    int32_t* pre3 = W + kWaitLists + 3 * A.cap;
    int r[4] = {0, 0, 0, 0};
    for (int base = 0; base < A.ccount; base += blockDim.x) {
      const int j = base + threadIdx.x;
      const int i = j < A.ccount ? A.corder[j] : -1;
      const bool w = i >= 0 && B.cluster_mode && B.flags[8 + i] == PH_PCG;
      const int kind = w ? B.inst[i].pcg_cluster : 0;
      const int pt3 = kind == 3 ? pcg_tiles(B, B.inst[i]) : 0;
      int v[4] = {kind == 1 ? 1 : 0, kind == 2 ? 1 : 0, kind == 3 ? 1 : 0, pt3}, t[4];
      block_scan4(v, t, scan_sm);
      if (kind >= 1 && kind <= 3) W[kWaitLists + (kind - 1) * A.cap + r[kind - 1] + v[kind - 1]] = i;
      if (kind == 3) pre3[r[2] + v[2] + 1] = r[3] + v[3] + pt3;
#pragma unroll
      for (int k = 0; k < 4; ++k) r[k] += t[k];
    }
    if (threadIdx.x == 0) {
      for (int k = 0; k < 3; ++k) {
        W[kWaitCount + k] = r[k];
        B.flags[4 + k] = r[k];
      }
      W[kWaitTake] = 0;
      W[kWaitTake + 1] = 0;
      W[kWaitLeft] = r[2];
      W[kWaitPass] = 0;
      W[kWaitDone] = 0;
      W[kWaitDone + 1] = 0;
      pre3[0] = 0;
    }
  }
  if (threadIdx.x == 0) {
    pt[0] = 0; pn[0] = 0; pl[0] = 0; pp[0] = 0;
    A.act[0] = run[0];
    B.flags[0] = run[0];
    const int alive = A.act[1];
    int need = max(max(run[1], run_pcg), max(run[2], run[3]));
    int p = min(alive, max(need, 1));
    A.act[1] = p;
    A.act[2] = min(p, eng_pcg_tiles);  // 0: no instance iterates its PCG in the engine
    A.act[3] = cluster_waiting;        // instances waiting for the cluster PCG kernel
    B.flags[1] = cluster_waiting;
  }
  __threadfence();
}

__device__ __forceinline__ void stage_clock(const EngineArgs& A, int kind, unsigned long long& t) {
  if (A.stage_ns && blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    A.stage_ns[kind] += now - t;
    A.stage_ns[16 + kind] += 1;
    t = now;
  }
}

__device__ __forceinline__ void engine_gave_up(const EngineArgs& A) {
  if (threadIdx.x == 0 && A.wait)
    for (int k = 0; k < 3; ++k) A.wait[kWaitCount + k] = 0;
  if (threadIdx.x == 0 && A.wait) A.wait[kWaitLeft] = 0;
}

template <typename Real>
__global__ void __launch_bounds__(kTile, (sizeof(Real) == 4 ? 3 : 2)) k_engine(BatchDev B, EngineArgs A) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  const int cta = blockIdx.x;
  int* ids = A.act + 4;
  int* pt = ids + A.cap;
  int* pn = pt + A.cap + 1;
  int* pl = pn + A.cap + 1;
  int* pp = pl + A.cap + 1;
  unsigned long long t = 0;
  if (A.stage_ns && cta == 0 && threadIdx.x == 0) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  // CTAs still running; the host sets act[1] = gridDim.x before the launch
  int alive = gridDim.x;
  int first_wait = -1;  // round in which an instance first waited for the cluster kernel
  // two barrier objects: the PCG group synchronises on its own counter while the CTAs
  // that skip the PCG block are already arriving at the next round-wide barrier
  // a CTA whose barrier wait gave up empties the waiting lists (no cluster PCG runs after a
  // failed launch) and leaves
#define PHX_SYNC(n, tag, kind)                                                                             \
  if (!grid_sync(A.bar, (unsigned)(n), tag, &A.bar->err, B.phase_live, A.wait_limit, A.unmet_tag == (tag))) { \
    engine_gave_up(A);                                                                                    \
    return;                                                                                               \
  }                                                                                                       \
  stage_clock(A, kind, t);
#define PHX_SYNC_PCG(n, tag, kind)                                                                  \
  if (!grid_sync(A.bar + 1, (unsigned)(n), tag, &A.bar->err, nullptr, A.wait_limit, A.unmet_tag == (tag))) { \
    engine_gave_up(A);                                                                             \
    return;                                                                                        \
  }                                                                                                \
  stage_clock(A, kind, t);
  // a stage (and the barrier after it) runs only if an instance is in its phase at the
  // last barrier's snapshot: every CTA reads the same snapshot, so all skip together
#define PHX_NEED(ph) (!B.phase_live || __ldcg(B.phase_live + 16 + (ph)) > 0)
  for (int r = 0; r < A.rounds; ++r) {
    if (cta == 0) compact(B, A);
    PHX_SYNC(alive, 1, K_CONTROL);
    const int na = __ldcg(A.act);
    if (na == 0) break;
    // hand over to the cluster PCG kernel once 1/wait_share of the active instances wait for
    // it, or wait_rounds rounds after the first one started waiting (the others keep going in
    // between: line-search trials and element passes do not need the cluster kernel)
    const int waiting = __ldcg(A.act + 3);
    if (waiting > 0 && first_wait < 0) first_wait = r;
    if (r > 0 && waiting > 0 && (A.wait_share * waiting >= na || r - first_wait >= A.wait_rounds)) break;
    // this round needs only P CTAs (P never grows within a launch: the rest leave)
    const int P = __ldcg(A.act + 1), Pp = __ldcg(A.act + 2);
    if (cta >= P) return;
    alive = P;
    const TileMap Mt{pt, ids, na}, Mn{pn, ids, na}, Ml{pl, ids, na}, Mp{pp, ids, na};
    if (PHX_NEED(PH_VEC)) {
      st_vecop(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 2, K_VECOP);
    }
    if (PHX_NEED(PH_EVAL)) {
      st_elem_eg(B, Mt, cta, P, sm, flag, smraw);
      PHX_SYNC(P, 3, K_ELEM_EG);
    }
    if (PHX_NEED(PH_EVAL)) {
      st_gather(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 4, K_GATHER);
    }
    if (PHX_NEED(PH_EVALK)) {
      st_elem_ek(B, Mt, cta, P, sm, flag);
      PHX_SYNC(P, 19, K_ELEM_EG);
    }
    if (PHX_NEED(PH_EVALK2)) {
      st_lin_ek(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 20, K_GATHER);
    }
    if (PHX_NEED(PH_VEC)) {
      st_vecop(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 5, K_VECOP);
    }
    if (PHX_NEED(PH_HESS)) {
      st_elem_hess<Real>(B, Mt, cta, P, sm, flag, smraw);
      PHX_SYNC(P, 6, K_ELEM_HESS);
    }
    if (PHX_NEED(PH_HESS)) {
      st_assemble<Real>(B, Ml, cta, P, sm, flag);
      PHX_SYNC(P, 7, K_ASSEMBLE);
    }
    if (PHX_NEED(PH_HESS) || PHX_NEED(PH_JACOBI)) {
      st_jacobi<Real>(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 8, K_JACOBI);
    }
    if (PHX_NEED(PH_LINSETUP)) {
      st_linsetup(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 9, K_LINSETUP);
    }
    if (PHX_NEED(PH_RESID)) {
      st_resid<Real>(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 10, K_RESID);
    }
    if (Pp > 0 && PHX_NEED(PH_PCG)) {
      if (cta < Pp) {
        // the PCG block only needs the CTAs that cover the node tiles
        for (int k = 0; k < A.pcg_chunk; ++k) {
          st_pcg_a<Real>(B, Mp, cta, Pp, sm, flag);
          PHX_SYNC_PCG(Pp, 11, K_PCG_A);
          st_pcg_b<Real>(B, Mp, cta, Pp, sm, flag);
          PHX_SYNC_PCG(Pp, 12, K_PCG_B);
        }
      }
      PHX_SYNC(P, 18, K_CONTROL);
    }
    if (PHX_NEED(PH_ACCUM)) {
      st_accum<Real>(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 13, K_ACCUM);
    }
    if (PHX_NEED(PH_RESID)) {
      st_resid<Real>(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 14, K_RESID);
    }
    if (PHX_NEED(PH_VEC)) {
      st_vecop(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 15, K_VECOP);
    }
    if (PHX_NEED(PH_EVAL)) {
      st_elem_eg(B, Mt, cta, P, sm, flag, smraw);
      PHX_SYNC(P, 16, K_ELEM_EG);
    }
    if (PHX_NEED(PH_EVAL)) {
      st_gather(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 17, K_GATHER);
    }
    if (PHX_NEED(PH_EVALK)) {
      st_elem_ek(B, Mt, cta, P, sm, flag);
      PHX_SYNC(P, 21, K_ELEM_EG);
    }
    if (PHX_NEED(PH_EVALK2)) {
      st_lin_ek(B, Mn, cta, P, sm, flag);
      PHX_SYNC(P, 22, K_GATHER);
    }
  }
#undef PHX_NEED
#undef PHX_SYNC
#undef PHX_SYNC_PCG
  if (cta == 0) compact(B, A);
}


// ---------------------------------------------------------------------------
// cluster PCG with rows in L2: k_pcg_cluster (phx_options.pcg_cluster = 2; the default,
// k_pcg_cg below, keeps the rows in shared memory)
// ---------------------------------------------------------------------------
// For instances up to kClusterMaxNodes nodes, the PCG iterations of a linear solve run
// inside one cluster of kCl CTAs: rows are split into contiguous chunk ranges, the two
// global reductions of an iteration go through distributed shared memory (every CTA
// sums the kCl partials in rank order, so all CTAs take the same decisions), and the
// iteration boundaries are hardware cluster barriers (barrier.cluster with
// release/acquire).  Vectors stay in global memory (L2-resident for these sizes);
// the rows another CTA wrote are read with ld.global.cg.
__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// The cluster's next position in a waiting list: thread 0 of rank 0 takes it from the list's
// counter and stores it into slot[par] of every CTA of the cluster; the cluster barrier
// publishes it.  Two slots, used in turn: a slot is written again only after every CTA has
// passed the barrier that follows its last read of it.  All CTAs get the same value.
template <int CL>
__device__ __forceinline__ int cl_next_job(int32_t* next, int* slot, unsigned& par) {
  if (cl_rank() == 0 && threadIdx.x == 0) {
    const int j = atomicAdd(next, 1);
    const unsigned a = (unsigned)__cvta_generic_to_shared(slot + par);
#pragma unroll
    for (unsigned r = 0; r < (unsigned)CL; ++r) {
      unsigned d;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(r));
      asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(d), "r"(j) : "memory");
    }
  }
  cl_sync();
  const int j = *(volatile int*)(slot + par);
  par ^= 1u;
  return j;
}
__device__ __forceinline__ double cl_ld(const double* local, unsigned rank) {
  unsigned src = (unsigned)__cvta_generic_to_shared(local), dst;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(dst) : "r"(src), "r"(rank));
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(dst) : "memory");
  return v;
}

__device__ __forceinline__ void ld4cg(const double* p, int64_t v, double (&o)[3]) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * v;
  double2 a = __ldcg(q), b = __ldcg(q + 1);
  o[0] = a.x; o[1] = a.y; o[2] = b.x;
}
__device__ __forceinline__ void ld4cg(const float* p, int64_t v, float (&o)[3]) {
  float4 a = __ldcg(reinterpret_cast<const float4*>(p) + v);
  o[0] = a.x; o[1] = a.y; o[2] = a.z;
}

// Sums K values over the CTA into v[] of thread 0 (fixed order: deterministic).
template <int K>
__device__ __forceinline__ void cta_sum256(double (&v)[K], double (*ws)[4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) ws[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += ws[w][k];
      v[k] = s;
    }
}

template <typename Real, int CL, int NT>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT) k_pcg_cluster(BatchDev B, const int32_t* list,
                                                                                const int32_t* countp, int32_t* next) {
  __shared__ double red[2][4];    // this CTA's partials, double-buffered by iteration
  __shared__ double ws[NT / 32][4];
  __shared__ double tot[4];
  __shared__ int jslot[2];
  const unsigned rank = cl_rank();
  const int count = __ldcg(countp);
  unsigned jpar = 0;
  cl_sync();  // every CTA of the cluster runs before rank 0 stores into their shared memory
  for (;;) {
    const int j = cl_next_job<CL>(next, jslot, jpar);
    if (j >= count) break;
    const int i = __ldcg(list + j);
    const InstDev I = B.inst[i];  // local copy: fields stay in registers across stores
    NState* st = I.st;
    if (I.pcg_cluster != 2 || *(volatile int32_t*)&st->phase != PH_PCG) continue;  // uniform over the cluster
    const int n = I.n, nch = I.nchunks;
    const int c0 = (int)(((int64_t)nch * rank) / CL), c1 = (int)(((int64_t)nch * (rank + 1)) / CL);
    const Real* H = PcgBufs<Real>::H(I);
    const Real* z = PcgBufs<Real>::z(I);
    Real* q = PcgBufs<Real>::q(I);
    Real* e = PcgBufs<Real>::e(I);
    Real* rv = PcgBufs<Real>::r(I);
    Real* zw = PcgBufs<Real>::z(I);
    const Real* Mi = PcgBufs<Real>::minv(I);
    const Real sh = (Real)st->shift;
    const double thr = st->thr_inner;
    const int maxit = I.opts->ls_num_max_iters;
    double rz = st->rz, beta = st->beta;
    int parity = st->pcg_parity, iter = st->pcg_iter, done_iters = 0, status = LIN_RUNNING, buf = 0;
    double rr = st->rr, pq = 0.0;
    while (true) {
      // q = (H + shift I) p, p = z + beta p_prev formed per column; p written for own rows
      const Real* pold = parity ? PcgBufs<Real>::pb(I) : PcgBufs<Real>::pa(I);
      Real* pnew = parity ? PcgBufs<Real>::pa(I) : PcgBufs<Real>::pb(I);
      const Real bt = (Real)beta;
      double pa_[1] = {0.0};
      {
        // L lanes per row: 4 when this CTA holds few rows (latency), 1 when it holds many
        const int r0 = c0 * 32, r1 = min(c1 * 32, n);
        const int rows = r1 - r0;
        auto sweep = [&](auto lanes_tag) {
          constexpr int L = decltype(lanes_tag)::value;
          const int sub = threadIdx.x & (L - 1), grp = threadIdx.x / L;
          for (int base = r0; base < r1; base += (int)(blockDim.x / L)) {
            const int v = base + grp;
            const bool valid = v < r1;
            Real acc[3];
            sell_row_lanes<L, Real, Real>(I, H, v, sub, valid,
                                          [&](int col, Real (&xc)[3]) {
                                            Real zc[3], pc[3];
                                            ld4cg(z, col, zc);
                                            ld4cg(pold, col, pc);
                                            for (int a = 0; a < 3; ++a) xc[a] = zc[a] + bt * pc[a];
                                          },
                                          acc);
            if (valid && sub == 0) {
              Real zv[3], pv[3];
              ld4cg(z, v, zv);
              ld4cg(pold, v, pv);
              for (int a = 0; a < 3; ++a) {
                pv[a] = zv[a] + bt * pv[a];
                acc[a] += sh * pv[a];
              }
              st4(pnew, v, pv);
              st4(q, v, acc);
              pa_[0] += (double)pv[0] * acc[0] + (double)pv[1] * acc[1] + (double)pv[2] * acc[2];
            }
          }
        };
        if (rows <= (int)blockDim.x / 4) sweep(std::integral_constant<int, 4>());
        else if (rows <= (int)blockDim.x / 2) sweep(std::integral_constant<int, 2>());
        else sweep(std::integral_constant<int, 1>());
      }
      cta_sum256<1>(pa_, ws);
      if (threadIdx.x == 0) red[buf][0] = pa_[0];
      cl_sync();
      if (threadIdx.x == 0) {
        double s = 0;
        for (unsigned r = 0; r < CL; ++r) s += cl_ld(&red[buf][0], r);
        tot[0] = s;
      }
      __syncthreads();
      pq = tot[0];
      bool last = false;
      double pq_use = pq;
      if (!(pq > 0.0)) {
        if (I.opts->curv_through && pq < 0.0) {
          // as Eigen's CG: a negative step along p, and on
        } else if (I.opts->precision != 0 && pq < 0.0 && iter == 0) {
          pq_use = -pq;  // truncated CG, first direction: step along p with |p.q| and stop
          last = true;
        } else {
          status = (I.opts->precision != 0 && pq < 0.0) ? LIN_TRUNCATED : LIN_BREAKDOWN;
          break;
        }
      }
      const Real alpha = (Real)(rz / pq_use);
      // e += alpha p, r -= alpha q, z = Minv r
      double pb_[2] = {0.0, 0.0};
      for (int v = c0 * 32 + (int)threadIdx.x; v < min(c1 * 32, n); v += (int)blockDim.x) {
        Real pv[3], qv[3], ev[3], rr_[3], zz[3];
        ld4(pnew, v, pv);
        ld4(q, v, qv);
        ld4(e, v, ev);
        ld4(rv, v, rr_);
        for (int a = 0; a < 3; ++a) {
          ev[a] += alpha * pv[a];
          rr_[a] -= alpha * qv[a];
        }
        for (int a = 0; a < 3; ++a)
          zz[a] = Mi[(size_t)(3 * a) * n + v] * rr_[0] + Mi[(size_t)(3 * a + 1) * n + v] * rr_[1] +
                  Mi[(size_t)(3 * a + 2) * n + v] * rr_[2];
        st4(e, v, ev);
        st4(rv, v, rr_);
        st4(zw, v, zz);
        pb_[0] += (double)rr_[0] * rr_[0] + (double)rr_[1] * rr_[1] + (double)rr_[2] * rr_[2];
        pb_[1] += (double)rr_[0] * zz[0] + (double)rr_[1] * zz[1] + (double)rr_[2] * zz[2];
      }
      cta_sum256<2>(pb_, ws);
      if (threadIdx.x == 0) {
        red[buf][1] = pb_[0];
        red[buf][2] = pb_[1];
      }
      cl_sync();
      if (threadIdx.x == 0) {
        double s1 = 0, s2 = 0;
        for (unsigned r = 0; r < CL; ++r) {
          s1 += cl_ld(&red[buf][1], r);
          s2 += cl_ld(&red[buf][2], r);
        }
        tot[1] = s1;
        tot[2] = s2;
      }
      __syncthreads();
      rr = tot[1];
      const double rzn = tot[2];
      ++iter;
      ++done_iters;
      buf ^= 1;
      if (last) {
        status = LIN_TRUNCATED;
        break;
      }
      if (rr < thr) {
        status = LIN_CONVERGED;
        break;
      }
      if (iter >= maxit) {
        status = LIN_MAXITER;
        break;
      }
      beta = rzn / rz;
      rz = rzn;
      parity ^= 1;
    }
    if (rank == 0 && threadIdx.x == 0) {
      st->pcg_iter = iter;
      st->pcg_total += done_iters;
      st->rr = rr;
      st->pq = pq;
      st->rz = rz;
      st->beta = beta;
      st->pcg_parity = parity;
      st->lin_status = status;
      st->phase = (status == LIN_BREAKDOWN) ? PH_LIN_DONE : PH_ACCUM;
      st->truncate = 0;
      if (B.algo_total)  // the same per-iteration bytes as the engine's spmv + pcg_update stages
        atomicAdd(B.algo_total + K_PCG_CLUSTER, (I.algo[K_PCG_A] + I.algo[K_PCG_B]) * done_iters);
      advance(B, i);
    }
    cl_sync();  // partial buffers are reused by the next instance
  }
}

// ---------------------------------------------------------------------------
// cluster PCG with shared-memory rows (FP32): k_pcg_cg
// ---------------------------------------------------------------------------
// The CG recurrence of A. T. Chronopoulos and C. W. Gear ("s-step iterative methods for
// symmetric linear systems", J. Comput. Appl. Math. 25 (1989)): with s = A z and the extra
// recurrence q = A p, all three inner products of an iteration are taken after its SpMV,
// so an iteration has one cluster barrier (z published) and one reduction:
//   p = z + b p, q = s + b q, e += a p, r -= a q, z = M^-1 r    (own rows, no exchange)
//   partials of gamma = (r, z), rho = (r, r)                     -> cluster barrier
//   s = (H + shift I) z  (z of other rows read from their CTA)   (own rows)
//   gamma, rho, delta = (z, s) summed over the cluster           -> one reduction
//   b = gamma / gamma_old, eta = delta - b gamma / a_old = (p, A p), a = gamma / eta
// In exact arithmetic these are the iterates of the two-reduction CG (Eigen's order); in
// floating point the variant is known to be about as accurate, unlike the pipelined forms,
// whose extra recurrences lose accuracy in FP32.  The convergence test on rho comes after
// the SpMV of the same iteration, which the converged iteration thus computes in vain; the
// sums and every decision are those of testing rho before it.
//
// Each of the CL CTAs owns contiguous SELL chunks.  Everything per row lives in its
// shared memory for the whole solve: z (read by the other CTAs through distributed shared
// memory, so the solve makes no global-memory exchange at all), r, e, p, s, q and the
// 3x3 block-Jacobi inverse; the matrix slices go to shared memory as far as they fit
// (chunk order), with the slot-row stride padded to 288 + 32/L floats so that the L lanes
// of a row hit different banks; later chunks are read from global memory.  z is
// overwritten only after the reduction, whose sums every CTA computes from its SpMV: no
// CTA reads the previous z any more.
constexpr int kCgSmem = 220 * 1024;  // dynamic shared memory per CTA of k_pcg_cg
constexpr int kCgMaxChunks = (kClusterMaxNodes + 31) / 32;
constexpr int kCgMaxCpc = (kCgMaxChunks + kCl - 1) / kCl;
static_assert(((4 * kCgMaxChunks + 15) & ~15) + ((4 * (kCgMaxCpc + 1) + 15) & ~15) + (6 * 16 + 9 * 4) * 32 * kCgMaxCpc <=
                  kCgSmem,
              "rows of the largest cluster instance must fit in shared memory");

constexpr int kLinAbort = -1;  // a reduction wait gave up: the cluster leaves together (cg_reduce)
constexpr int kLinYield = -2;  // the solve's time slice ended: its state is saved, it resumes in a later launch
// A solve leaves its cluster at the end of an iteration (a time slice) once it has iterated
// slice_min times in this launch, at least one solve of the launch has ended, and enough of the
// launch's clusters found no solve left (slice_share x idle >= clusters): the instances whose
// solves ended then go on in the engine while this one waits for the next cluster launch,
// where it resumes from the saved state with the same bits.
struct CgResult {  // FP32 like the solve; widened once when written to the instance state
  int iter, done, status;
  float rr, eta, gamma, beta, alpha;
};
// Dynamic shared memory of k_pcg_cg, declared at file scope so that the helpers below form
// their pointers from it: the compiler then knows every one of them is shared and issues
// shared-memory loads and stores, rather than generic ones through the pointers of a struct.
extern __shared__ __align__(16) unsigned char cg_smem[];
template <typename T>
__device__ __forceinline__ T* cgs(uint32_t off) {
  return reinterpret_cast<T*>(cg_smem + off);
}

struct CgShared {  // per-CTA layout (byte offsets into cg_smem), the same in every CTA of the cluster
  uint32_t tab;                // u32[nch] distributed-shared address of each chunk's z rows
  uint32_t co;                 // i32[cpc + 1] own chunk offsets (slots)
  uint32_t z, r, e, p, s, q;   // float4[mrows]
  uint32_t mi;                 // f32[9][mrows] block-Jacobi inverses, plane-major
  uint32_t hs, cs;             // own matrix slices (chunks c0 .. csplit-1), slot-row strides hst, cst
  int mrows;                   // rows of every vector array (32 per owned chunk slot)
  int hst, cst, csplit;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t cl_map(uint32_t a, unsigned rank) {
  uint32_t d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(rank));
  return d;
}
__device__ __forceinline__ float4 cl_ld4f(uint32_t a) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(a));
  return v;
}

// Cluster-wide sums of K <= 3 FP32 partials: warp shuffles, one __syncthreads, then lanes
// 0..CL-1 of warp 0 push the CTA's sums with st.async into slot [rank] of every CTA, each
// store completing bytes on the receiving CTA's mbarrier; every thread waits for its own
// mbarrier's phase and adds the CL slots in rank order (the same sums, hence the same
// decisions, everywhere).  No cluster barrier and no fence: the slots carry only the sums,
// and the mbarrier makes them visible.  FP32 throughout: this part has a small fraction of
// FP32's FP64 rate, and the PCG accumulates in FP32 by design (the FP64 residual of the
// refinement sweep decides).
//
// Reuse of the single slot buffer, ws and the mbarrier needs no barrier of its own: a CTA
// pushes the sums of the next reduction only after the cluster barrier that follows its
// next update, which every CTA reaches only after reading this reduction's slots; warp 0
// reads ws before its push, which every wait depends on.
//
// The wait gives up after kCgWaitCycles.  The decision is made uniform before any CTA
// leaves, because a peer may still push into this CTA's slots or read its z rows:
//  * within the CTA: __syncthreads_or over the threads' own waits, so all of them agree;
//  * within the cluster: the CTA that gave up stores 1 into the abort word of every CTA
//    of the cluster (its own included) and flags the batch error, then goes on to the
//    next cluster barrier, the same one its peers reach next (an iteration's, or the end
//    of the instance's; all CTAs pass the same barriers up to that point because their
//    decisions come from the same sums).  The barrier's release/acquire makes the abort
//    word visible to every CTA after it; each checks it right after each barrier that can
//    follow a reduction and, if set, drains its own mbarrier (cg_drain: bounded) and
//    returns, so no CTA touches another's shared memory after that barrier.
constexpr long long kCgWaitCycles = 2000000000LL;
constexpr long long kCgDrainCycles = 200000000LL;  // pushes in flight into this CTA at an abort
// fl (thread 0's value) travels in the fourth float of the CTA's push; every CTA reads rank 0's
// as red[0][3] once the reduction has landed, so a decision that rank 0 takes is the same in
// every CTA.
template <int K, int CL, int NT>
__device__ __forceinline__ bool cg_reduce(float (&p)[K], unsigned rank, float (*red)[4], float (*ws)[4], uint32_t mbar,
                                          unsigned& phase, int32_t* err, uint32_t abort_sm, float (&tot)[K],
                                          float fl = 0.f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) p[k] += __shfl_down_sync(0xffffffffu, p[k], off);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) ws[warp][k] = p[k];
  __syncthreads();
  if (warp == 0) {
    float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < K; ++k) {
      v[k] = lane < NT / 32 ? ws[lane][k] : 0.f;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
      v[k] = __shfl_sync(0xffffffffu, v[k], 0);
    }
    v[3] = __shfl_sync(0xffffffffu, fl, 0);
    if (lane == 0)
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(CL * 16) : "memory");
    if (lane < CL) {
      const uint32_t dst = cl_map(smem_u32(&red[rank][0]), (unsigned)lane);
      const uint32_t mb = cl_map(mbar, (unsigned)lane);
      asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];"
                   ::"r"(dst), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "r"(mb)
                   : "memory");
    }
  }
  const unsigned parity = phase & 1u;
  ++phase;
  const long long t0 = clock64();
  int gave_up = 0;
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) break;
    if (clock64() - t0 > kCgWaitCycles) {
      gave_up = 1;
      break;
    }
  }
  if (__syncthreads_or(gave_up)) {  // the whole CTA gives up; tell every CTA of the cluster
    if (threadIdx.x < CL) {
      const uint32_t dst = cl_map(abort_sm, threadIdx.x);
      asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(dst), "r"(1) : "memory");
    }
    if (threadIdx.x == 0) atomicExch(err, 1);
    return false;
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float s = 0.f;
#pragma unroll
    for (int r = 0; r < CL; ++r) s += red[r][k];
    tot[k] = s;
  }
  return true;
}

// The abort word of this CTA (set by any CTA of the cluster that gave up a wait), read after
// a cluster barrier: the same value in every thread and every CTA.
__device__ __forceinline__ bool cg_aborted(uint32_t abort_sm) {
  uint32_t v;
  asm volatile("ld.volatile.shared::cta.u32 %0, [%1];" : "=r"(v) : "r"(abort_sm) : "memory");
  return v != 0u;
}

// Before leaving after an abort: waits (bounded) for the phase of the last reduction to
// complete, so that no push of a peer is still on its way into this CTA's shared memory.
__device__ __forceinline__ void cg_drain(uint32_t mbar, unsigned phase) {
  if (threadIdx.x == 0 && phase > 0) {
    const unsigned parity = (phase - 1u) & 1u;
    const long long t0 = clock64();
    for (;;) {
      uint32_t done;
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(done)
          : "r"(mbar), "r"(parity)
          : "memory");
      if (done || clock64() - t0 > kCgDrainCycles) break;
    }
  }
  __syncthreads();
}

// The slots k = sub, sub + L, ... < len of one row (lane `lane` of its chunk) from slot-row
// R0 on, accumulated into acc: four slots at a time per lane, their column ids and blocks
// loaded together, then the z gathers (own rows from this CTA's shared memory, other rows
// through distributed shared memory), then the arithmetic.  SM: the slices are in shared
// memory (stride hst, cst; planes 0-3 and 4-7 of a slot-row as one float4 per lane, then
// plane 8); otherwise in global memory (stride 288, 32; plane after plane), read-only.
template <int L, bool SM>
__device__ __forceinline__ void cg_row(const float* hb, const int* cb, int hst, int cst, int R0, int len, int lane,
                                       int sub, const float4* Z, const uint32_t* tab, int row0, int nrow,
                                       float (&acc)[3]) {
  for (int k0 = sub; k0 < len; k0 += 4 * L) {
    int col[4];
    float h[4][9];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int k = k0 + u * L;
      const bool in = k < len;
      const int R = R0 + (in ? k : 0);
      if (SM) {  // planes 0-3 and 4-7 as float4 per lane, then plane 8
        col[u] = in ? cb[R * cst + lane] : -1;
        const float* hr = hb + R * hst;
        const float4 a = in ? reinterpret_cast<const float4*>(hr)[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 b = in ? reinterpret_cast<const float4*>(hr + 128)[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        h[u][0] = a.x; h[u][1] = a.y; h[u][2] = a.z; h[u][3] = a.w;
        h[u][4] = b.x; h[u][5] = b.y; h[u][6] = b.z; h[u][7] = b.w;
        h[u][8] = in ? hr[256 + lane] : 0.f;
      } else {
        const float* hp = hb + (size_t)R * hst + lane;
        col[u] = in ? __ldg(cb + (size_t)R * cst + lane) : -1;
#pragma unroll
        for (int q = 0; q < 9; ++q) h[u][q] = in ? __ldg(hp + q * 32) : 0.f;
      }
    }
    float4 x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int cc = col[u];
      const unsigned lr = (unsigned)(cc - row0);
      if (cc < 0) x[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      else if (lr < (unsigned)nrow) x[u] = Z[lr];
      else x[u] = cl_ld4f(tab[cc >> 5] + ((uint32_t)(cc & 31) << 4));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      acc[0] += h[u][0] * x[u].x + h[u][1] * x[u].y + h[u][2] * x[u].z;
      acc[1] += h[u][3] * x[u].x + h[u][4] * x[u].y + h[u][5] * x[u].z;
      acc[2] += h[u][6] * x[u].x + h[u][7] * x[u].y + h[u][8] * x[u].z;
    }
  }
}

// s = (H + shift I) z for the CTA's rows, L lanes per row, and the partial (z, s): two
// dependent round trips per four slots of a lane.
template <int L, int NT>
__device__ __forceinline__ float cg_spmv(const InstDev& I, const CgShared& S, int c0, int row0, int row1, int64_t sb,
                                         float sh) {
  const int sub = threadIdx.x & (L - 1), grp = threadIdx.x / L, nrow = row1 - row0;
  const float4* Z = cgs<const float4>(S.z);
  float4* Sv = cgs<float4>(S.s);
  const int* co = cgs<const int>(S.co);
  const uint32_t* tab = cgs<const uint32_t>(S.tab);
  float part = 0.f;
  for (int base = row0; base < row1; base += NT / L) {
    const int v = base + grp;
    const bool ok = v < row1;
    float acc[3] = {0.f, 0.f, 0.f};
    if (ok) {
      const int c = v >> 5, lane = v & 31;
      const int s0 = co[c - c0], len = (co[c - c0 + 1] - s0) >> 5;
      const int R0 = (int)((s0 - sb) >> 5);
      if (c < S.csplit)
        cg_row<L, true>(cgs<const float>(S.hs), cgs<const int>(S.cs), S.hst, S.cst, R0, len, lane, sub, Z, tab, row0,
                        nrow, acc);
      else
        cg_row<L, false>(I.H32 + (sb >> 5) * 288, I.slot_col + sb, 288, 32, R0, len, lane, sub, Z, tab, row0, nrow,
                         acc);
    }
#pragma unroll
    for (int off = 1; off < L; off <<= 1)
#pragma unroll
      for (int a = 0; a < 3; ++a) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], off);
    if (ok && sub == 0) {
      const float4 z = Z[v - row0];
      const float4 s = make_float4(acc[0] + sh * z.x, acc[1] + sh * z.y, acc[2] + sh * z.z, 0.f);
      Sv[v - row0] = s;
      part += z.x * s.x + z.y * s.y + z.z * s.z;
    }
  }
  return part;
}

// One linear solve (the inner PCG of one refinement sweep) of instance I in this cluster.
// Scalars and inner products in FP32; the results go back to the FP64 state.
template <int L, int CL, int NT>
__device__ __forceinline__ CgResult cg_solve(const InstDev& I, const CgShared& S, unsigned rank, int c0, int row0,
                                          int row1, int64_t sb, float (*red)[4], float (*ws)[4], uint32_t mbar,
                                          unsigned& phase, int32_t* err, uint32_t abort_sm, float sh, float thr,
                                          int maxit, bool trunc_ok, int iter0, bool resume, const int32_t* slice,
                                          int ncl, int slice_share, int slice_min) {
  const int nrow = row1 - row0, ms = S.mrows;
  float4* const Z = cgs<float4>(S.z);
  float4* const Rv = cgs<float4>(S.r);
  float4* const Ev = cgs<float4>(S.e);
  float4* const Pv = cgs<float4>(S.p);
  float4* const Sv = cgs<float4>(S.s);
  float4* const Qv = cgs<float4>(S.q);
  const float* const Mi = cgs<const float>(S.mi);
  CgResult out{iter0, 0, LIN_RUNNING, 0.f, 0.f, 0.f, 0.f, 0.f};
  float gam, eta, beta, alpha;
  bool last = false;
  if (resume) {
    // the state the last time slice saved: this CTA's rows of r, z, e, p, s, q and the
    // scalars of the next iteration, the exact FP32 values
    for (int t = threadIdx.x; t < nrow; t += NT) {
      const int v = row0 + t;
      float r[3], z[3], e[3], p[3], s[3], q[3];
      ld4(I.r32, v, r);
      ld4(I.z32, v, z);
      ld4(I.e32, v, e);
      ld4(I.p32a, v, p);
      ld4(I.p32b, v, s);
      ld4(I.q32, v, q);
      Rv[t] = make_float4(r[0], r[1], r[2], 0.f);
      Z[t] = make_float4(z[0], z[1], z[2], 0.f);
      Ev[t] = make_float4(e[0], e[1], e[2], 0.f);
      Pv[t] = make_float4(p[0], p[1], p[2], 0.f);
      Sv[t] = make_float4(s[0], s[1], s[2], 0.f);
      Qv[t] = make_float4(q[0], q[1], q[2], 0.f);
    }
    const NState* st = I.st;
    gam = (float)st->rz;
    eta = (float)st->pq;
    beta = (float)st->beta;
    alpha = (float)st->alpha;
    out.rr = (float)st->rr;
    out.eta = eta;
    out.gamma = gam;
    out.beta = beta;
    __syncthreads();  // the first iteration's vector update reads only this CTA's rows
  } else {
    // start: r and z = M^-1 r from the residual stage, e = 0
    float g1[2] = {0.f, 0.f};
    for (int t = threadIdx.x; t < nrow; t += NT) {
      float r[3], z[3];
      ld4(I.r32, row0 + t, r);
      ld4(I.z32, row0 + t, z);
      Rv[t] = make_float4(r[0], r[1], r[2], 0.f);
      Z[t] = make_float4(z[0], z[1], z[2], 0.f);
      Ev[t] = make_float4(0.f, 0.f, 0.f, 0.f);
      g1[0] += r[0] * z[0] + r[1] * z[1] + r[2] * z[2];
      g1[1] += r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    }
    cl_sync();  // z of every CTA written
    float p3[3] = {g1[0], g1[1], cg_spmv<L, NT>(I, S, c0, row0, row1, sb, sh)};
    float t3[3];
    if (!cg_reduce<3, CL, NT>(p3, rank, red, ws, mbar, phase, err, abort_sm, t3)) {
      cl_sync();  // the barrier the peers reach next; they see the abort word after it
      out.status = kLinAbort;
      return out;
    }
    gam = t3[0];
    out.rr = t3[1];
    if (t3[1] < thr) {
      out.status = LIN_CONVERGED;
      return out;
    }
    eta = t3[2];
    beta = 0.f;
    out.eta = eta;
    out.gamma = gam;
    if (!(eta > 0.f)) {
      if (!trunc_ok && eta < 0.f) {
        // Eigen's ConjugateGradient has no curvature test: a negative step along p, and on
      } else if (trunc_ok && eta < 0.f && out.iter == 0) {
        eta = -eta;  // truncated CG, first direction: one step along z with |z.Az| and stop
        last = true;
      } else {
        out.status = (trunc_ok && eta < 0.f) ? LIN_TRUNCATED : LIN_BREAKDOWN;
        return out;
      }
    }
    alpha = gam / eta;
  }
  for (int it = 0;; ++it) {
    if (out.iter >= maxit) {
      out.status = LIN_MAXITER;
      break;
    }
    const float a = alpha, b = beta;
    const bool first = it == 0 && !resume;
    // rank 0 decides whether this iteration ends the solve's time slice; the decision reaches
    // every CTA with this iteration's reduction
    float slice_fl = 0.f;
    if (slice && rank == 0 && threadIdx.x == 0 && it + 1 >= slice_min) {
      const int ended = *(volatile const int32_t*)slice, idle = *(volatile const int32_t*)(slice + 1);
      if (ended > 0 && slice_share * idle >= ncl) slice_fl = 1.f;
    }
    float g[2] = {0.f, 0.f};
    for (int t = threadIdx.x; t < nrow; t += NT) {
      const float4 z = Z[t], s = Sv[t];
      float4 p = first ? z : Pv[t], q = first ? s : Qv[t];
      if (!first) {
        p = make_float4(z.x + b * p.x, z.y + b * p.y, z.z + b * p.z, 0.f);
        q = make_float4(s.x + b * q.x, s.y + b * q.y, s.z + b * q.z, 0.f);
      }
      float4 e = Ev[t];
      e.x += a * p.x;
      e.y += a * p.y;
      e.z += a * p.z;
      Ev[t] = e;
      if (last) continue;
      float4 r = Rv[t];
      r.x -= a * q.x;
      r.y -= a * q.y;
      r.z -= a * q.z;
      const float* m = Mi + t;
      const float zx = m[0] * r.x + m[ms] * r.y + m[2 * ms] * r.z;
      const float zy = m[3 * ms] * r.x + m[4 * ms] * r.y + m[5 * ms] * r.z;
      const float zz = m[6 * ms] * r.x + m[7 * ms] * r.y + m[8 * ms] * r.z;
      Pv[t] = p;
      Qv[t] = q;
      Rv[t] = r;
      Z[t] = make_float4(zx, zy, zz, 0.f);
      g[0] += r.x * zx + r.y * zy + r.z * zz;
      g[1] += r.x * r.x + r.y * r.y + r.z * r.z;
    }
    ++out.iter;
    ++out.done;
    if (last) {
      out.status = LIN_TRUNCATED;
      break;
    }
    cl_sync();  // the new z of every CTA written; none reads the previous z any more
    if (cg_aborted(abort_sm)) {  // a CTA gave up the last reduction: leave together
      out.status = kLinAbort;
      return out;
    }
    float pg[3] = {g[0], g[1], cg_spmv<L, NT>(I, S, c0, row0, row1, sb, sh)};
    float tg[3];
    if (!cg_reduce<3, CL, NT>(pg, rank, red, ws, mbar, phase, err, abort_sm, tg, slice_fl)) {
      cl_sync();  // the barrier the peers reach next; they see the abort word after it
      out.status = kLinAbort;
      return out;
    }
    const bool slice_end = red[0][3] != 0.f;  // rank 0's decision, the same in every CTA
    const float gam_new = tg[0];
    out.rr = tg[1];
    if (tg[1] < thr) {
      out.status = LIN_CONVERGED;
      break;
    }
    beta = gam_new / gam;
    eta = tg[2] - beta * gam_new / alpha;
    gam = gam_new;
    out.eta = eta;
    out.gamma = gam;
    out.beta = beta;
    if (!(eta > 0.f) && !(!trunc_ok && eta < 0.f)) {  // not positive definite along p (or non-finite)
      out.status = (trunc_ok && eta < 0.f) ? LIN_TRUNCATED : LIN_BREAKDOWN;
      break;
    }
    alpha = gam / eta;
    if (slice_end) {
      // the slice ends: the rows go to the instance's FP32 vectors (s in p32b), the scalars
      // to its state (written by the caller); the next launch resumes with the same bits
      for (int t = threadIdx.x; t < nrow; t += NT) {
        const int v = row0 + t;
        const float4 r = Rv[t], z = Z[t], e = Ev[t], p = Pv[t], sv = Sv[t], q = Qv[t];
        st4(I.r32, v, {r.x, r.y, r.z});
        st4(I.z32, v, {z.x, z.y, z.z});
        st4(I.e32, v, {e.x, e.y, e.z});
        st4(I.p32a, v, {p.x, p.y, p.z});
        st4(I.p32b, v, {sv.x, sv.y, sv.z});
        st4(I.q32, v, {q.x, q.y, q.z});
      }
      out.alpha = alpha;
      out.status = kLinYield;
      break;
    }
  }
  return out;
}

// slice: [0] solves of this launch that ended, [1] clusters that found no solve left (the
// time slices read them; null: every solve runs to its end).  A solve's slice ends after at
// least slice_min iterations in this launch, once a solve ended and slice_share x the idle
// clusters reach the launch's cluster count.
template <int CL, int NT>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT, 1) k_pcg_cg(BatchDev B, const int32_t* list,
                                                                               const int32_t* countp, int32_t* next,
                                                                               int32_t* slice, int slice_share,
                                                                               int slice_min) {
  __shared__ __align__(16) float red[CL][4];  // partial sums pushed by every CTA of the cluster
  __shared__ float ws[NT / 32][4];
  __shared__ __align__(8) uint64_t mbar_obj;   // completes when all CL pushes of a reduction landed
  __shared__ uint32_t abort_word;              // set by a CTA of the cluster that gave up a wait
  const unsigned rank = cl_rank();
  const int tid = threadIdx.x;
  const uint32_t mbar = smem_u32(&mbar_obj);
  const uint32_t abort_sm = smem_u32(&abort_word);
  unsigned phase = 0;  // reductions waited for so far (the mbarrier's phase)
  if (tid == 0) {
    abort_word = 0u;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  cl_sync();  // every mbarrier initialised before any CTA pushes to it
  int32_t* err = B.flags + 2;
  __shared__ int jslot[2];
  const int count = __ldcg(countp);
  unsigned jpar = 0;
  const int ncl = (int)(gridDim.x / CL);
  for (;;) {
    const int j = cl_next_job<CL>(next, jslot, jpar);
    if (j >= count) {
      if (slice && rank == 0 && tid == 0) atomicAdd(slice + 1, 1);
      break;
    }
    const int i = __ldcg(list + j);
    const InstDev& I = B.inst[i];  // fields are re-read (L1) where needed: registers go to the rows
    NState* st = I.st;
    if (I.pcg_cluster != 1 || *(volatile int32_t*)&st->phase != PH_PCG) continue;  // uniform over the cluster
    const bool resume = *(volatile int32_t*)&st->pcg_resume != 0;  // written before this launch: uniform
    const int n = I.n, nch = I.nchunks;
    const int cpc = (nch + CL - 1) / CL;
    const int c0 = min(nch, (int)rank * cpc), c1 = min(nch, c0 + cpc);
    const int row0 = c0 * 32, row1 = max(row0, min(c1 * 32, n)), nrow = row1 - row0;
    const int mrows = 32 * cpc;
    const int L = nrow <= NT / 4 ? 4 : (nrow <= NT / 2 ? 2 : 1);
    // shared layout: tab u32[nch] | co i32[cpc+1] | z r e p s q float4[mrows] | mi f32[9][mrows] | matrix
    CgShared S;
    uint32_t off = 0;
    S.tab = off;
    off += (4u * nch + 15u) & ~15u;
    S.co = off;
    off += (4u * (cpc + 1) + 15u) & ~15u;
    S.z = off;
    S.r = S.z + 16u * mrows;
    S.e = S.r + 16u * mrows;
    S.p = S.e + 16u * mrows;
    S.s = S.p + 16u * mrows;
    S.q = S.s + 16u * mrows;
    off = S.q + 16u * mrows;
    S.mi = off;
    S.mrows = mrows;
    off += 36u * mrows;
    off = (off + 15u) & ~15u;
    uint32_t* tab = cgs<uint32_t>(S.tab);
    int* co = cgs<int>(S.co);
    float* mi = cgs<float>(S.mi);
    const int64_t sb = __ldg(I.chunk_off + c0);
    // matrix slices of chunks c0 .. csplit-1 in shared memory, slot-row stride padded per L
    const int pad = L == 1 ? 0 : 32 / L;
    S.hst = 288 + pad;
    S.cst = 32 + pad;
    const int64_t per_row = (int64_t)4 * (S.hst + S.cst);  // bytes per slot-row of 32 slots
    const int64_t room = (int64_t)kCgSmem - off;
    int csplit = c0;
    while (csplit < c1 && (int64_t)((__ldg(I.chunk_off + csplit + 1) - sb) >> 5) * per_row <= room) ++csplit;
    S.csplit = csplit;
    const int nsr = (int)((__ldg(I.chunk_off + csplit) - sb) >> 5);  // slot-rows held in shared memory
    S.hs = off;
    S.cs = off + 4u * S.hst * nsr;
    float* hs = cgs<float>(S.hs);
    int* cs = cgs<int>(S.cs);
    // fill: chunk table, chunk offsets, inverses, matrix slices
    const uint32_t zloc = smem_u32(cgs<float4>(S.z));
    for (int c = tid; c < nch; c += NT) {
      const int owner = c / cpc;
      tab[c] = cl_map(zloc, (unsigned)owner) + (uint32_t)((c - owner * cpc) * 32 * 16);
    }
    for (int c = tid; c <= c1 - c0; c += NT) co[c] = __ldg(I.chunk_off + c0 + c);
    for (int k = tid; k < 9 * nrow; k += NT) {
      const int plane = k / nrow, t = k - plane * nrow;
      mi[plane * mrows + t] = __ldg(I.minv32 + (size_t)plane * n + row0 + t);
    }
    {
      const float* hg = I.H32 + (sb >> 5) * 288;
      const int* cg = I.slot_col + sb;
      // slot-row layout in shared memory: planes 0-3 as one float4 per lane, planes 4-7 as
      // one float4 per lane, plane 8 (the global layout holds the nine planes one after
      // the other): a slot's block is three loads, the same bytes
      for (int k = tid; k < nsr * 32; k += NT) {
        const int R = k >> 5, l = k & 31;
        const float* src = hg + (size_t)R * 288 + l;
        float q[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) q[e] = __ldg(src + 32 * e);
        float* dst = hs + (size_t)R * S.hst;
        reinterpret_cast<float4*>(dst)[l] = make_float4(q[0], q[1], q[2], q[3]);
        reinterpret_cast<float4*>(dst + 128)[l] = make_float4(q[4], q[5], q[6], q[7]);
        dst[256 + l] = q[8];
      }
      for (int k = tid; k < nsr * 8; k += NT) {  // 32 ids = 8 int4 per slot-row
        const int R = k >> 3, w = k & 7;
        reinterpret_cast<int4*>(cs + (size_t)R * S.cst)[w] = __ldg(reinterpret_cast<const int4*>(cg + (size_t)R * 32) + w);
      }
    }
    __syncthreads();
    const float sh = (float)st->shift;
    const float thr = (float)st->thr_inner;
    const int maxit = I.opts->ls_num_max_iters;
    // FP32 path at negative curvature: truncate (Steihaug), or go on as Eigen's CG does
    const bool trunc_ok = I.opts->precision != 0 && !I.opts->curv_through;
    const int iter0 = st->pcg_iter;
    CgResult out;
    if (L == 4) out = cg_solve<4, CL, NT>(I, S, rank, c0, row0, row1, sb, red, ws, mbar, phase, err, abort_sm, sh, thr, maxit,
                                           trunc_ok, iter0, resume, slice, ncl, slice_share, slice_min);
    else if (L == 2) out = cg_solve<2, CL, NT>(I, S, rank, c0, row0, row1, sb, red, ws, mbar, phase, err, abort_sm, sh, thr, maxit,
                                           trunc_ok, iter0, resume, slice, ncl, slice_share, slice_min);
    else out = cg_solve<1, CL, NT>(I, S, rank, c0, row0, row1, sb, red, ws, mbar, phase, err, abort_sm, sh, thr, maxit,
                                           trunc_ok, iter0, resume, slice, ncl, slice_share, slice_min);
    if (out.status == kLinAbort) {  // every CTA of the cluster leaves after the same barrier
      cg_drain(mbar, phase);
      return;                       // the batch error is flagged; the host reports a timeout
    }
    if (out.status == kLinYield) {
      // the rows are saved; the instance keeps waiting for the cluster PCG (phase PH_PCG)
      if (rank == 0 && tid == 0) {
        st->pcg_iter = out.iter;
        st->pcg_total += out.done;
        st->rr = out.rr;
        st->pq = out.eta;
        st->rz = out.gamma;
        st->beta = out.beta;
        st->alpha = out.alpha;
        st->pcg_resume = 1;
        st->pcg_slices++;
        if (B.algo_total)
          atomicAdd(B.algo_total + K_PCG_CLUSTER, (I.algo[K_PCG_A] + I.algo[K_PCG_B]) * out.done);
      }
      cl_sync();  // shared buffers and partial slots are reused by the next instance
      if (cg_aborted(abort_sm)) {
        cg_drain(mbar, phase);
        return;
      }
      continue;
    }
    for (int t = tid; t < nrow; t += NT) {
      const float4 e = cgs<float4>(S.e)[t];
      const float ev[3] = {e.x, e.y, e.z};
      st4(I.e32, row0 + t, ev);
    }
    if (rank == 0 && tid == 0) {
      if (slice) atomicAdd(slice, 1);
      st->pcg_resume = 0;
      st->pcg_iter = out.iter;
      st->pcg_total += out.done;
      st->rr = out.rr;
      st->pq = out.eta;
      st->rz = out.gamma;
      st->beta = out.beta;
      st->pcg_parity = 0;
      st->lin_status = out.status;
      st->phase = (out.status == LIN_BREAKDOWN) ? PH_LIN_DONE : PH_ACCUM;
      st->truncate = 0;
      if (B.algo_total)  // the same per-iteration bytes as the engine's spmv + pcg_update stages
        atomicAdd(B.algo_total + K_PCG_CLUSTER, (I.algo[K_PCG_A] + I.algo[K_PCG_B]) * out.done);
      advance(B, i);
    }
    cl_sync();  // shared buffers and partial slots are reused by the next instance
    if (cg_aborted(abort_sm)) {  // a CTA gave up the solve's last reduction: leave together
      cg_drain(mbar, phase);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename Real>
size_t hess_smem() { return (size_t)kTile * 90 * sizeof(Real); }

cudaError_t setup_kernel_attributes() {
  cudaError_t e = cudaFuncSetAttribute(k_elem_hess<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)hess_smem<double>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_elem_hess<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hess_smem<float>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_engine<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hess_smem<double>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_engine<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hess_smem<float>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_pcg_cg<kCl, kClThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, kCgSmem);

  return e;
}

int engine_grid(bool fp64, int num_sms) {
  int nb = 0;
  cudaError_t e = fp64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_engine<double>, kTile, hess_smem<double>())
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_engine<float>, kTile, hess_smem<float>());
  if (e != cudaSuccess || nb < 1) return 0;
  return nb * num_sms;
}

// Before an engine launch (one thread): both grid barriers cleared and the round's CTA count.
__global__ void k_prep(BatchDev B, EngineArgs A, int grid) {
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 2; ++k) A.bar[k] = GridBar{0u, 0u, 0, 0};
  A.act[0] = 0;
  A.act[1] = grid;
}

// End of one pass of the graph's solve loop (one thread): go on while instances are active and
// no bounded wait gave up, for at most loop_cap passes.
__global__ void k_loop_end(BatchDev B, EngineArgs A, cudaGraphConditionalHandle h, int32_t* loops, int loop_cap) {
  if (threadIdx.x != 0) return;
  const bool failed = A.bar[0].err || A.bar[1].err || B.flags[2];
  const int pass = ++loops[0];
  cudaGraphSetConditional(h, (!failed && B.flags[0] > 0 && pass < loop_cap) ? 1u : 0u);
}

cudaError_t launch_prep(cudaStream_t s, const BatchDev& B, const EngineArgs& A, int grid) {
  k_prep<<<1, 32, 0, s>>>(B, A, grid);
  return cudaGetLastError();
}

// The waiting list, its count and its take counter for cluster PCG kind 1 or 2 (one place for
// the host launch and the graph).
struct ClusterArgs {
  const int32_t* list;
  const int32_t* count;
  int32_t* take;
  int32_t* slice;  // kind 1: the counters its time slices read
};
ClusterArgs cluster_args(int32_t* wait, int cap, int kind) {
  return ClusterArgs{wait + kWaitLists + (kind - 1) * cap, wait + kWaitCount + (kind - 1), wait + kWaitTake + (kind - 1),
                     wait + kWaitDone};
}

cudaError_t launch_pcg_cluster(cudaStream_t s, const BatchDev& B, int32_t* wait, int cap, int clusters, int kind,
                               int slice_share, int slice_min) {
  if (clusters <= 0) return cudaSuccess;
  const ClusterArgs c = cluster_args(wait, cap, kind);
  const int32_t* list = c.list;
  const int32_t* count = c.count;
  int32_t* take = c.take;
  if (kind == 1)
    k_pcg_cg<kCl, kClThreads><<<clusters * kCl, kClThreads, kCgSmem, s>>>(B, list, count, take,
                                                                          slice_share > 0 ? c.slice : nullptr,
                                                                          slice_share, slice_min);
  else k_pcg_cluster<float, kCl, kClThreads><<<clusters * kCl, kClThreads, 0, s>>>(B, list, count, take);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// whole-GPU PCG of the FP32 instances above the cluster size (PCG kind 3)
// ---------------------------------------------------------------------------
// The engine's two PCG stages as kernels of their own, so that they run at the occupancy of
// a small kernel (the engine holds 12 warps per SM) and the kernel boundary is the grid-wide
// synchronisation.  Tiles, partial sums and decisions are the engine's (the instance's own
// tile width, per-tile partials summed in tile order), so an instance gets the bits it gets
// when the engine iterates its PCG.
constexpr int kGpcgBlocks = 6;  // resident CTAs per SM the whole-GPU PCG kernels are built for (24 warps)

__device__ __forceinline__ TileMap gpcg_map(const EngineArgs& A) {
  const int32_t* W = A.wait;
  return TileMap{W + kWaitLists + 3 * A.cap, W + kWaitLists + 2 * A.cap, __ldcg(W + kWaitCount + 2)};
}

__global__ void __launch_bounds__(kTile, kGpcgBlocks) k_gpcg_a(BatchDev B, EngineArgs A) {
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_pcg_a<float, true>(B, gpcg_map(A), blockIdx.x, gridDim.x, sm, flag, A.wait + kWaitLeft);
}

__global__ void __launch_bounds__(kTile, kGpcgBlocks) k_gpcg_b(BatchDev B, EngineArgs A) {
  __shared__ double sm[32 * 5];
  __shared__ int flag;
  st_pcg_b<float, true>(B, gpcg_map(A), blockIdx.x, gridDim.x, sm, flag, A.wait + kWaitLeft);
}

// graph form: the loop runs while a kind-3 instance iterates (at most cap passes per launch)
__global__ void k_gpcg_begin(EngineArgs A, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0) return;
  A.wait[kWaitPass] = 0;
  cudaGraphSetConditional(h, A.wait[kWaitLeft] > 0 ? 1u : 0u);
}
__global__ void k_gpcg_loop(EngineArgs A, cudaGraphConditionalHandle h, int cap) {
  if (threadIdx.x != 0) return;
  A.cfg[2]++;  // iterations of the graph's kind-3 loops since the host last cleared it
  const int pass = ++A.wait[kWaitPass];
  cudaGraphSetConditional(h, (A.wait[kWaitLeft] > 0 && pass < cap) ? 1u : 0u);
}

int gpcg_grid(int num_sms) {
  int na = 0, nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&na, k_gpcg_a, kTile, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gpcg_b, kTile, 0) != cudaSuccess) {
    cudaGetLastError();
    return num_sms;
  }
  return std::max(1, std::min(na, nb)) * num_sms;
}

cudaError_t launch_gpcg(cudaStream_t s, const BatchDev& B, const EngineArgs& A, int grid, int pairs,
                        cudaEvent_t* ev) {
  for (int k = 0; k < pairs; ++k) {
    if (ev) cudaEventRecord(ev[4 * k], s);
    k_gpcg_a<<<grid, kTile, 0, s>>>(B, A);
    if (ev) cudaEventRecord(ev[4 * k + 1], s);
    if (ev) cudaEventRecord(ev[4 * k + 2], s);
    k_gpcg_b<<<grid, kTile, 0, s>>>(B, A);
    if (ev) cudaEventRecord(ev[4 * k + 3], s);
  }
  return cudaGetLastError();
}

int max_active_clusters(int kind) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kCl * 256);
  cfg.blockDim = dim3(kClThreads);
  cfg.dynamicSmemBytes = kind == 1 ? kCgSmem : 0;
  int n = 0;
  cudaError_t e = kind == 1 ? cudaOccupancyMaxActiveClusters(&n, (const void*)k_pcg_cg<kCl, kClThreads>, &cfg)
                            : cudaOccupancyMaxActiveClusters(&n, (const void*)k_pcg_cluster<float, kCl, kClThreads>, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

namespace {
cudaError_t add_kernel(cudaGraph_t g, cudaGraphNode_t* node, cudaGraphNode_t* dep, const void* fn, dim3 grid,
                       dim3 block, size_t smem, void** args) {
  cudaKernelNodeParams p = {};
  p.func = const_cast<void*>(fn);
  p.gridDim = grid;
  p.blockDim = block;
  p.sharedMemBytes = (unsigned)smem;
  p.kernelParams = args;
  return cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &p);
}
}  // namespace

cudaError_t build_solve_graph(bool fp64, int grid, const BatchDev& B, const EngineArgs& A,
                              const int clusters[2], int gpcg, int32_t* loops, int loop_cap, cudaGraph_t* graph,
                              cudaGraphExec_t* exec) {
  *graph = nullptr;
  *exec = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  cudaGraphNode_t cnode;
  cudaGraphNodeParams cp = {};
  e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&cnode, g, nullptr, nullptr, 0, &cp);
  }
  // kernel arguments are copied when the nodes are added
  BatchDev b = B;
  EngineArgs a = A;
  int gr = grid, cap = loop_cap;
  int32_t* lp = loops;
  cudaGraphNode_t prev = nullptr, node = nullptr;
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    void* pa[] = {&b, &a, &gr};
    e = add_kernel(body, &node, nullptr, (const void*)k_prep, dim3(1), dim3(32), 0, pa);
    prev = node;
    if (e == cudaSuccess) {
      void* ea[] = {&b, &a};
      const void* fn = fp64 ? (const void*)k_engine<double> : (const void*)k_engine<float>;
      e = add_kernel(body, &node, &prev, fn, dim3(grid), dim3(kTile), fp64 ? hess_smem<double>() : hess_smem<float>(),
                     ea);
      if (e == cudaSuccess) {
        cudaLaunchAttributeValue v = {};
        v.cooperative = 1;
        e = cudaGraphKernelNodeSetAttribute(node, cudaLaunchAttributeCooperative, &v);
      }
      prev = node;
    }
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      if (clusters[k] <= 0) continue;
      const ClusterArgs c = cluster_args(A.wait, A.cap, k + 1);
      const int32_t* list = c.list;
      const int32_t* countp = c.count;
      int32_t* next = c.take;
      int32_t* slice = A.slice_share > 0 ? c.slice : nullptr;
      int share = A.slice_share, smin = A.slice_min;
      void* ca[] = {&b, &list, &countp, &next, &slice, &share, &smin};  // k_pcg_cluster takes the first four
      const void* fn = k == 0 ? (const void*)k_pcg_cg<kCl, kClThreads> : (const void*)k_pcg_cluster<float, kCl, kClThreads>;
      e = add_kernel(body, &node, &prev, fn, dim3(clusters[k] * kCl), dim3(kClThreads), k == 0 ? kCgSmem : 0, ca);
      prev = node;
    }
    if (gpcg > 0 && e == cudaSuccess) {
      // the kind-3 PCG: a while-loop inside the pass, its condition set by k_gpcg_begin and
      // k_gpcg_loop (at most loop_cap iterations before the engine runs again)
      cudaGraphConditionalHandle gh;
      cudaGraphNodeParams gp = {};
      e = cudaGraphConditionalHandleCreate(&gh, g, 0, 0);
      if (e == cudaSuccess) {
        void* ba[] = {&a, &gh};
        e = add_kernel(body, &node, &prev, (const void*)k_gpcg_begin, dim3(1), dim3(32), 0, ba);
        prev = node;
      }
      if (e == cudaSuccess) {
        gp.type = cudaGraphNodeTypeConditional;
        gp.conditional.handle = gh;
        gp.conditional.type = cudaGraphCondTypeWhile;
        gp.conditional.size = 1;
        e = cudaGraphAddNode(&node, body, &prev, nullptr, 1, &gp);
        prev = node;
      }
      if (e == cudaSuccess) {
        cudaGraph_t inner = gp.conditional.phGraph_out[0];
        cudaGraphNode_t n1, n2, n3;
        void* ka[] = {&b, &a};
        e = add_kernel(inner, &n1, nullptr, (const void*)k_gpcg_a, dim3(gpcg), dim3(kTile), 0, ka);
        if (e == cudaSuccess) e = add_kernel(inner, &n2, &n1, (const void*)k_gpcg_b, dim3(gpcg), dim3(kTile), 0, ka);
        int icap = 1 << 20;
        void* la2[] = {&a, &gh, &icap};
        if (e == cudaSuccess) e = add_kernel(inner, &n3, &n2, (const void*)k_gpcg_loop, dim3(1), dim3(32), 0, la2);
      }
    }
    if (e == cudaSuccess) {
      void* la[] = {&b, &a, &h, &lp, &cap};
      e = add_kernel(body, &node, &prev, (const void*)k_loop_end, dim3(1), dim3(32), 0, la);
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
  if (e != cudaSuccess) {
    if (*exec) cudaGraphExecDestroy(*exec);
    *exec = nullptr;
    cudaGraphDestroy(g);
    return e;
  }
  *graph = g;
  return cudaSuccess;
}

cudaError_t launch_engine(bool fp64, int grid, cudaStream_t s, const BatchDev& B, const EngineArgs& A) {
  BatchDev b = B;
  EngineArgs a = A;
  void* args[] = {(void*)&b, (void*)&a};
  if (fp64)
    return cudaLaunchCooperativeKernel((const void*)k_engine<double>, dim3(grid), dim3(kTile), args,
                                       hess_smem<double>(), s);
  return cudaLaunchCooperativeKernel((const void*)k_engine<float>, dim3(grid), dim3(kTile), args, hess_smem<float>(),
                                     s);
}

void launch(KernelId id, int grid, cudaStream_t s, const BatchDev& B, bool fp64) {
  if (grid <= 0) return;
  switch (id) {
    case K_ELEM_EG: k_elem_eg<<<grid, kTile, 3 * kTileNodeCap * sizeof(double), s>>>(B); break;
    case K_GATHER: k_gather<<<grid, kTile, 0, s>>>(B); break;
    case K_ELEM_HESS:
      if (fp64) k_elem_hess<double><<<grid, kTile, hess_smem<double>(), s>>>(B);
      else k_elem_hess<float><<<grid, kTile, hess_smem<float>(), s>>>(B);
      break;
    case K_ASSEMBLE:
      if (fp64) k_assemble<double><<<grid, kTile, 0, s>>>(B); else k_assemble<float><<<grid, kTile, 0, s>>>(B);
      break;
    default: break;  // the other stages run only inside k_engine
  }
}

const char* kernel_name(KernelId id) {
  switch (id) {
    case K_CONTROL: return "control";
    case K_VECOP: return "vecop";
    case K_ELEM_EG: return "elem_eg";
    case K_GATHER: return "gather";
    case K_ELEM_HESS: return "elem_hess";
    case K_ASSEMBLE: return "assemble";
    case K_JACOBI: return "jacobi";
    case K_LINSETUP: return "linsetup";
    case K_RESID: return "resid";
    case K_PCG_A: return "spmv";
    case K_PCG_B: return "pcg_update";
    case K_ACCUM: return "accum";
    case K_PCG_CLUSTER: return "pcg_cluster";
    case K_ENGINE: return "engine";
    default: return "?";
  }
}

}  // namespace phx
