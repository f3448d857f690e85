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

cudaError_t setup_kernel_attributes();
void launch(KernelId id, int grid, cudaStream_t s, const BatchDev& B, bool fp64);
const char* kernel_name(KernelId id);

}  // namespace phx
