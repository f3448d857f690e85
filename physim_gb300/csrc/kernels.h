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
  long long wait_limit;  // SM cycles a grid-barrier wait lasts before it gives up
  int unmet_tag;         // test hook: the grid barrier with this tag waits for one arrival more than
                         // the CTAs taking part, so it gives up (0: none)
};
constexpr long long kBarrierLimit = 4000000000LL;  // default wait_limit: about 2 s of SM clock

cudaError_t setup_kernel_attributes();
int engine_grid(bool fp64, int num_sms);
cudaError_t launch_engine(bool fp64, int grid, cudaStream_t s, const BatchDev& B, const EngineArgs& A);
// PCG of every listed instance that is in PH_PCG, one cluster per instance
cudaError_t launch_pcg_cluster(cudaStream_t s, const BatchDev& B, const int32_t* list, int count, int kind);
// One stage as its own kernel, for the evaluation entry points: K_ELEM_EG, K_GATHER,
// K_ELEM_HESS or K_ASSEMBLE (other ids launch nothing; their stages run inside k_engine)
void launch(KernelId id, int grid, cudaStream_t s, const BatchDev& B, bool fp64);
const char* kernel_name(KernelId id);

}  // namespace phx
