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
  K_COUNT
};
static_assert(K_COUNT <= 12, "InstDev::algo holds 12 kernel kinds");

// Grid barrier state of the engine (device memory, zeroed before a launch).
struct GridBar {
  unsigned int arrive, gen;
  int err;    // set when a barrier wait gave up
  int stage;  // which barrier timed out
};

struct EngineArgs {
  GridBar* bar;
  int32_t* act;                   // [1 + cap + 3 (cap + 1)]: count, ids, tet/node/lob tile prefixes
  unsigned long long* stage_ns;   // [32]: ns per stage kind, then executions per kind; or null
  int cap;
  int rounds;
  int pcg_chunk;
};

cudaError_t setup_kernel_attributes();
int engine_grid(bool fp64, int num_sms);
cudaError_t launch_engine(bool fp64, int grid, cudaStream_t s, const BatchDev& B, const EngineArgs& A);
void launch(KernelId id, int grid, cudaStream_t s, const BatchDev& B, bool fp64);
const char* kernel_name(KernelId id);

}  // namespace phx
