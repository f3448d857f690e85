// kernels.h -- launch interface of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "phx_types.h"

namespace phx {

enum KernelId : int {
  K_CONTROL = 0,
  K_VECOP,
  K_ELEM_EG,
  K_GATHER,
  K_ELEM_HESS,
  K_ASSEMBLE,
  K_JACOBI,
  K_LINSETUP,
  K_RESID,
  K_PCG_A,
  K_PCG_B,
  K_ACCUM,
  K_PCG_CLUSTER,
  K_ENGINE,  // whole engine launches (profiling events only; no bytes)
  K_COUNT
};
static_assert(K_COUNT <= 16, "InstDev::algo holds 16 kernel kinds");

// Grid barrier state of the engine (device memory, zeroed before a launch).
struct GridBar {
  unsigned int arrive, gen;
  int err;    // set when a barrier wait gave up
  int stage;  // which barrier timed out
};

struct EngineArgs {
  GridBar* bar;                   // [2]: round-wide barrier, PCG-block barrier
  int32_t* act;                   // [4 + cap + 4 (cap + 1)]: count, CTAs in the round, CTAs in the
                                  // PCG block, cluster solves waiting; ids; tet/node/lob/PCG tile prefixes
  unsigned long long* stage_ns;   // [32]: ns per stage kind, then executions per kind; or null
  int cap;
  int rounds;
  int pcg_chunk;
  int wait_rounds;  // hand the waiting instances to the cluster PCG kernel this many rounds after the
  int wait_share;   // first one waited, or once waiting * wait_share >= active
  int slice_share;  // cluster-PCG time slices (phx_launch_settings::slice_share, slice_min)
  int slice_min;
  long long wait_limit;  // SM cycles a grid-barrier wait lasts before it gives up
  int unmet_tag;         // test hook: the grid barrier with this tag waits for one arrival more than
                         // the CTAs taking part, so it gives up (0: none)
  int32_t* cfg;          // [4]: [1] graph loop passes, [2] iterations of the graph's kind-3 PCG loops
  const int32_t* corder; // [ccount] batch positions of the cluster-PCG instances, largest first
  int ccount;
  int32_t* wait;         // [wait_size(cap)]: instances waiting for the cluster and grid PCG kernels
                         // (layout below; written by the engine at the end of each launch)
};
// Layout of EngineArgs::wait: at kWaitCount the waiting counts of PCG kinds 1..3 (1, 2: one
// cluster per instance, 3: the whole-GPU kernels k_gpcg_a/b); at kWaitTake the take counters
// of kinds 1 and 2; at kWaitLeft the kind-3 instances still iterating; at kWaitPass the kind-3
// loop's passes; at kWaitDone the kind-1 solves that ended in this cluster launch and at
// kWaitDone + 1 its clusters that found no solve left (what a solve's time slice reads); from
// kWaitLists the three lists (cap each, corder's order) and the kind-3 PCG tile prefix (cap + 1).
constexpr int kWaitCount = 0, kWaitTake = 3, kWaitLeft = 5, kWaitPass = 6, kWaitDone = 7, kWaitLists = 10;
inline int wait_size(int cap) { return kWaitLists + 4 * cap + 1; }
constexpr long long kBarrierLimit = 4000000000LL;  // default wait_limit: about 2 s of SM clock

cudaError_t setup_kernel_attributes();
int engine_grid(bool fp64, int num_sms);
cudaError_t launch_engine(bool fp64, int grid, cudaStream_t s, const BatchDev& B, const EngineArgs& A);
// Before each engine launch: barrier state cleared and the round's CTA count
cudaError_t launch_prep(cudaStream_t s, const BatchDev& B, const EngineArgs& A, int grid);
// PCG of the instances the engine listed as waiting for PCG kind `kind` (1: rows in shared
// memory, 2: rows in L2): `clusters` clusters take them in list order until none is left
cudaError_t launch_pcg_cluster(cudaStream_t s, const BatchDev& B, int32_t* wait, int cap, int clusters, int kind,
                               int slice_share, int slice_min);
// Clusters of PCG kind `kind` that fit on the device at once (0 if the query fails)
int max_active_clusters(int kind);
// The whole-GPU PCG of the FP32 instances of kind 3 (above the cluster size): `pairs` PCG
// iterations (k_gpcg_a: p update + SpMV + p.q; k_gpcg_b: vector update + r.r, r.z) over the
// instances the engine listed; an instance that leaves its PCG is skipped from then on and
// counted off wait[kWaitLeft].  grid: CTAs of 128 threads (gpcg_grid).
int gpcg_grid(int num_sms);
cudaError_t launch_gpcg(cudaStream_t s, const BatchDev& B, const EngineArgs& A, int grid, int pairs,
                        cudaEvent_t* ev = nullptr);
// The whole solve loop as one graph: while instances are active, k_prep, k_engine, the cluster
// PCG kernels (clusters[k] clusters of kind k + 1; 0 leaves it out) and k_loop_end, which sets
// the loop condition from the engine's flags (no instance active, a barrier or cluster wait gave
// up, or loop_cap passes) and counts the passes in loops[0].
// gpcg > 0 adds the kind-3 loop (k_gpcg_begin, then while instances iterate: k_gpcg_a,
// k_gpcg_b, k_gpcg_loop) with gpcg CTAs per kernel.
cudaError_t build_solve_graph(bool fp64, int grid, const BatchDev& B, const EngineArgs& A,
                              const int clusters[2], int gpcg, int32_t* loops, int loop_cap, cudaGraph_t* graph,
                              cudaGraphExec_t* exec);
// One stage as its own kernel, for the evaluation entry points: K_ELEM_EG, K_GATHER,
// K_ELEM_HESS or K_ASSEMBLE (other ids launch nothing; their stages run inside k_engine)
void launch(KernelId id, int grid, cudaStream_t s, const BatchDev& B, bool fp64);
const char* kernel_name(KernelId id);

// A field of one instance sampled on the cell centres of a grid over its rest shape (field.cu).
struct GridSampleArgs {
  int n, m;
  const int32_t* tets;   // [m][4]
  const double* xrest;   // [n][4] rest positions
  const double* x;       // [n][4] positions
  const double* energy;  // [m] element energies (field 5), else unused
  int field;             // PHX_FIELD_*
  int shape[3];
  double origin[3], delta[3];
  double fill;
  int32_t* owner;        // [cells] owning tet or -1
  double* values;        // [cells]
};
// k_grid_init, k_grid_claim (one warp per tet), k_grid_eval (one thread per cell) on stream s.
cudaError_t launch_grid_sample(cudaStream_t s, const GridSampleArgs& a, int num_sms);

}  // namespace phx
