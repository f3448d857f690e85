// phx_types.h -- device-resident data layout of one instance and of a batch.
//
// Layout in HBM, per instance (all buffers 256-byte aligned, from the context arena):
//   tets        int4 [m]            node ids
//   rest64      double[m][12]       Dm^-1 (col-major 9), w = rest volume, lambda, mu
//   rest32      float [m][12]       same in FP32 (FP32 Hessian kernel)
//   model       uint8 [m]
//   node vectors double4 [n]        x, xs (saved state), dx, g, gn, dxprev, x0, v0, v, hlin
//   SELL-32 3x3 block matrix        chunks of 32 rows, each padded to its longest row;
//                                   slot s, entry e lives at vals[(s>>5)*288 + e*32 + (s&31)]
//   lower-block tables              lo_slot / up_slot / seg_ptr / seg_c (scatter map)
//   node tables                     nseg_ptr / nseg_c (gradient gather), fixmask, mass
//   PCG vectors (Real = float|double, 4-wide per node): r, z, p[2], q, e; Minv [9][n]
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define PHX_HD __host__ __device__
#include <vector_types.h>
#else
#define PHX_HD
#endif

namespace phx {

constexpr int kTile = 128;       // tets / nodes / lower blocks per tile
constexpr int kChunk = 32;       // SELL chunk height (one warp)
constexpr int kPartials = 8;     // doubles reduced per tile (at most)
constexpr int kCl = 8;           // CTAs per cluster of the cluster PCG
constexpr int kClThreads = 512;  // threads per CTA of the cluster PCG
constexpr int kOneChunkTiles = 608;  // instances up to this many SELL chunks take one-chunk PCG tiles (else four)
constexpr int kClusterMaxNodes = 13000;  // instances up to this size solve their PCG in one cluster
constexpr int kWaitRounds = 4;           // engine rounds an instance may wait for the cluster kernel
constexpr int kWaitShare = 2;            // ... or until 1/kWaitShare of the active instances wait
constexpr int kSliceShare = 2;           // cluster-PCG time slices end once half the launch's clusters are idle ...
constexpr int kSliceMin = 32;            // ... and the solve iterated this often in the launch

// Phases of the per-instance Newton state machine (see control in kernels.cu).
enum Phase : int32_t {
  PH_DONE = 0,
  PH_START = 1,       // control: begin SolveFull
  PH_VEC = 2,         // node-parallel vector op pending (vecop flags), then next_phase
  PH_EVAL = 3,        // device: energy + gradient at x
  PH_EVAL_DONE = 4,   // control
  PH_ITER = 5,        // control: start of SolveStepInternal
  PH_HESS = 6,        // device: element Hessian + assembly + Jacobi
  PH_JACOBI = 7,      // device: Jacobi only (new regularisation shift)
  PH_LINSETUP = 8,    // device: b = -g, dx = guess
  PH_RESID = 9,       // device: r = b - (H + s I) dx in FP64, inner rhs
  PH_PCG = 10,        // device: PCG iterations
  PH_ACCUM = 11,      // device: dx += e, norms
  PH_LIN_DONE = 12,   // control: regularisation checks, clamp, line search start
  PH_EVALK = 13,      // device: element energies at several line-search trial steps
  PH_EVALK2 = 14,     // device: their linear-load (and inertia) energies, then the scan
};
constexpr int kLsK = 8;  // most line-search trial steps evaluated together

enum VecOp : int32_t {
  VO_RESTORE = 1,     // x = xs
  VO_ACCEPT = 2,      // g = gn ; dxprev = alpha * dx
  VO_SAVE = 4,        // xs = x
  VO_STEEP = 8,       // dx = -g
  VO_TRIAL = 16,      // x = xs + alpha * dx
  VO_VEL = 32,        // v = (x - x0) / dt
  VO_PRED = 64,       // x0 = x ; v0 = v ; x = x0 + dt * v0
  VO_GCOPY = 128,     // g = gn
  VO_ZERODX = 256,    // dx = 0
  VO_BACK = 512,     // keep the saved iterate as the restart point of an FP64 finish
  VO_STAGE = 1024,   // staged boundary conditions: targets (and soft stiffness) of the current stage
  VO_GNEW = 2048,    // g = gn (re-evaluation at the start of an iteration)
};

// LIN_TRUNCATED: the FP32 path met negative curvature and kept the iterate so far
// (truncated CG).  The plain path goes on through negative curvature, as Eigen's CG does;
// LIN_BREAKDOWN is p.q = 0 or a non-finite value, and regularises like a result with b.x < 0.
enum LinStatus : int32_t { LIN_RUNNING = 0, LIN_CONVERGED = 1, LIN_MAXITER = 2, LIN_BREAKDOWN = 3, LIN_TRUNCATED = 4 };

enum DevError : int32_t { DEV_OK = 0, DEV_NONFINITE = 1, DEV_BADSTATE = 2 };

// Solver options as the device sees them (host phx_options, resolved).
struct DevOpts {
  int32_t qp_solver, min_step_max_count, min_impr_max_count, num_max_iters, try_steepest;
  int32_t ls_num_max_iters, ls_num_reg_trials, lsearch_num_try, precision, precond;
  int32_t max_refine_sweeps, warm_guess, dynamic, ls_parallel;  // ls_parallel: trials evaluated together
  int32_t lsearch_type, pad_o;                                   // LSearchType: 0 None .. 4 WolfeStrong
  double tol_max_error, tol_min_step, tol_min_impr, max_step_size, ls_tol_max_error;
  double lsearch_alpha, inner_tol, dt, tol_rel;
  double lsearch_wolfe1, lsearch_wolfe2;                         // Armijo / Wolfe constants c1, c2
  int32_t num_stages, stage_values;  // staged loading: stages until fully constrained (0, 1: none);
                                     // 1 if a stage changes targets or stiffness (re-evaluate)
  int32_t curv_through, pad_cv;      // FP32 PCG at negative curvature: 1 goes on like Eigen's CG
};

// Scalar state of one instance's solve (one thread of the control kernel owns it).
struct NState {
  int32_t phase, next_phase, vecop, purpose;   // purpose: 0 init eval, 1 line-search eval
  int32_t result, it, steepest, min_impr_count;
  int32_t min_step_count, num_bis, total_bis, reg_trial;
  int32_t total_reg, sweeps, total_sweeps, lin_status;
  int32_t pcg_iter, pcg_parity, error, first_step;
  int32_t step_result, nofix, hess_count, truncate;
  int64_t pcg_total;
  double obj, opt, opt0, obj_new;
  double alpha_trial, factor, scale, dx_norm;
  double b_dot_dx, E_el, E_eval, gg_eval;
  double normA2, shift, regT, bb;
  double rr64, rz, rr, pq;
  double alpha, beta, thr_inner, thr_final;
  double tol_eff;                              // max(tol_max_error, tol_rel * opt0)
  double lin_tol;                              // relative residual target of this step's linear solve
  double eta, opt_prev;                        // forcing term state (FP32 path)
  double log_step;                             // ||dx_final|| of the step being logged
  double dg, dg_eval;                          // dx . g at the search's start; dx . g at the trial
  int32_t log_pending, log_count;              // per-iteration log bookkeeping
  int32_t lsk;                                 // trials in the batch being evaluated (PH_EVALK)
  int32_t pcg_resume;                          // 1: the cluster PCG left its solve at a time slice's end, state saved
  double ls_a[8], ls_e[8], ls_eel[8];          // their step lengths, energies, element energies
  int32_t stage, iter_staged;                  // boundary-condition stage; 1 once this iteration stepped it
  int32_t pcg_slices, pad_sl;                  // cluster-PCG time slices that ended before their solve
};

constexpr int kLogCap = 256;                   // Newton iterations kept in the per-instance log

// Device descriptor of one instance (pointers into the arena).
struct InstDev {
  int32_t n, m, nlo, nchunks;
  int64_t nslots;
  int32_t pcg_cluster;         // PCG inside one cluster: 0 no, 1 shared-memory rows (k_pcg_cg), 2 rows in L2 (k_pcg_cluster)
  int32_t pad_c;
  // mesh + rest data
  const int32_t* tets;        // [m][4]
  const double* rest64;       // [m][12]
  const float* rest32;        // [m][12]
  const int32_t* tile_nptr;   // [tiles(m)+1] unique nodes of each tet tile, ascending ...
  const int32_t* tile_nodes;  // ... concatenated
  const uint16_t* tet_loc;    // [m][4] each corner's index in its tile's node list
  const uint8_t* model;       // [m]
  // pattern / scatter map
  const int32_t* chunk_off;   // [nchunks+1] slot offsets (multiples of 32)
  const int32_t* slot_col;    // [nslots]
  const int32_t* diag_slot;   // [n]
  const int32_t* lo_rc;       // [nlo][2] (R, C)
  const int32_t* lo_slot;     // [nlo]
  const int32_t* up_slot;     // [nlo], -1 on the diagonal
  const int32_t* seg_ptr;     // [nlo+1]
  const int32_t* seg_c;       // [10m] e*10 + p, grouped by lower block, element order
  const int32_t* nseg_ptr;    // [n+1]
  const int32_t* nseg_c;      // [4m] e*4 + a, grouped by node, element order
  const uint8_t* fixmask;     // [n] bit d = DoF d fixed
  const double* mass;         // [n] lumped mass per node
  double* hlin;               // [n][4] f - m g : linear-load term of energy and gradient
  double* soft;               // [n][4] soft fixed position (target x, y, z, stiffness k) per node, or null
  const int32_t* stage_grp;   // [n] staged group of each node (-1: none), or null
  const double* stage_ini;    // [n][4] the start value its targets are animated from
  const double* stage_par;    // [groups][16]: num_stages, soft, k_start, k_end, move (9, row-major), shift (3)
  // FP64 node vectors [n][4]
  const double* xrest;
  double* x; double* xs; double* dx; double* g; double* gn; double* dxprev;
  double* xback;              // the accepted iterate one Newton step before xs (FP64 finish restarts there)
  double* x0; double* v0; double* v; double* r64; double* bvec;
  // element scratch
  double* Eloc;               // [m]
  double* Gloc;               // [m][12]
  float* Hloc32;              // [m][90]
  double* Hloc64;             // [m][90]
  // matrix values (SELL)
  float* H32;                 // [nslots*9]
  double* H64;
  // PCG vectors, Real = float / double, 4-wide per node
  float* r32; float* z32; float* p32a; float* p32b; float* q32; float* e32; float* minv32;
  double* rd; double* zd; double* pda; double* pdb; double* qd; double* ed; double* minvd;
  // reductions
  double* partials;           // [max tiles][kPartials]
  uint32_t* counter;          // [1]
  NState* st;
  const DevOpts* opts;
  double* log;                // [kLogCap][4]: obj, opt, bisections, step per Newton iteration
  double algo[16];            // algorithmic bytes of one launch of each kernel kind on this instance
};

// Tile prefix arrays of the active batch (device memory).
struct BatchDev {
  const int32_t* num;         // [1] active instances
  const int32_t* pre_tet;     // [num+1]
  const int32_t* pre_node;
  const int32_t* pre_lob;
  InstDev* inst;              // [num]
  int32_t* flags;             // [8 + num]: [0] active count, [1] cluster solves waiting, [2] a cluster
                              // PCG wait gave up; [8 + i] phase of instance i
  double* algo_total;         // [16] algorithmic bytes summed per kernel kind, or null
  int32_t* phase_live;        // [32] active instances per phase bucket: [0..15] kept current by
                              // advance(), [16..31] the copy taken at the last grid barrier, or null
  int32_t cluster_mode;       // 1: instances with pcg_cluster leave their PCG to k_pcg_cluster
};

constexpr int kBucketClusterPcg = 15;  // phase bucket of instances waiting for the cluster PCG kernel

PHX_HD inline int64_t sell_addr(int64_t s, int e) { return (s >> 5) * 288 + (int64_t)e * 32 + (s & 31); }

}  // namespace phx
