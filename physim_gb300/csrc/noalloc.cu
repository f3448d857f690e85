// noalloc.cu -- element Hessian + assembly for callers that cannot allocate device memory.
//
// Who needs this: a host application that hands this library its device buffers but does
// not let it allocate -- a physics or game engine that reserves all GPU memory in its own
// pool at start-up, an embedding runtime that forbids cudaMalloc once frames are running
// (cudaMalloc/cudaFree can synchronise the whole device and stall other work), or a
// caller whose memory is accounted by a foreign allocator.  Every other entry point of the
// library works on an instance whose buffers live in the context's arena, which is
// allocated with cudaMalloc.  This one takes device pointers for all of its inputs and
// its output and keeps its only scratch -- the 10 oriented 3x3 blocks of every tet,
// before they are summed -- in a fixed, file-scope device array.
//
// The array is PHX_NOALLOC_MAX_TETS * 90 doubles (about 23.6 MB) and every GPU that loads
// the library holds it until the process exits.  Larger meshes are rejected.  Calls share
// the array: two calls whose kernels overlap on the GPU (different streams, or different
// host threads on one device) race on it, so a caller serialises them (one stream).  A
// call overwrites every scratch entry it later reads, so nothing has to start at zero and
// the contents a previous call left behind are never used.
//
// Host code must not pass the array's name to a kernel: in host code it is only a
// stand-in for the device symbol.  Its device address is looked up once per device with
// cudaGetSymbolAddress, on the first call made while that device is current; that first
// call therefore has to happen before any stream capture that would record this entry
// point.  The address is kept per device index for the life of the process: the entry
// point assumes the device's primary context throughout (after cudaDeviceReset the kept
// address would be stale).  Indices are trusted (tets < num_nodes, seg_c < 10 num_tets),
// as the header states; the kernels do not check them.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/phx.h"
#include "element.cuh"
#include "errors.h"

namespace {

constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_hloc[(size_t)PHX_NOALLOC_MAX_TETS * 90];

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

int fail(int code, const std::string& msg) { return phx::set_last_error(code, msg); }

// Device address of the scratch array on the current device (looked up once per device).
int scratch_for_current_device(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PHX_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PHX_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_hloc);
    if (e != cudaSuccess || !p)
      return fail(PHX_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return PHX_OK;
}

// One thread per tet: the 10 lower-oriented node blocks into the scratch rows.
__global__ void __launch_bounds__(128) k_noalloc_elem(int m, const int32_t* __restrict__ tets,
                                                      const double* __restrict__ rest,
                                                      const uint8_t* __restrict__ model,
                                                      const double* __restrict__ x, const double* __restrict__ X0,
                                                      double* __restrict__ scratch) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  int nd[4];
  for (int a = 0; a < 4; ++a) nd[a] = tets[4 * (size_t)e + a];
  double u0[3];
  for (int r = 0; r < 3; ++r) u0[r] = x[3 * (size_t)nd[0] + r] - X0[3 * (size_t)nd[0] + r];
  double Du[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r)
      Du[r + 3 * c] = (x[3 * (size_t)nd[c + 1] + r] - X0[3 * (size_t)nd[c + 1] + r]) - u0[r];
  const double* r64 = rest + 12 * (size_t)e;
  phx::elem_blocks_core<double>(nd, Du, r64, r64, model ? model[e] : 0, scratch + 90 * (size_t)e);
}

// One thread per (lower block, entry): the block's contributions summed in element order.
__global__ void __launch_bounds__(288) k_noalloc_assemble(int nlo, const int32_t* __restrict__ seg_ptr,
                                                          const int32_t* __restrict__ seg_c,
                                                          const double* __restrict__ scratch,
                                                          double* __restrict__ out) {
  const int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = it / 9;
  const int ent = (int)(it % 9);
  if (k >= nlo) return;
  double s = 0.0;
  for (int c = seg_ptr[k]; c < seg_ptr[k + 1]; ++c) s += scratch[(size_t)seg_c[c] * 9 + ent];
  out[9 * k + ent] = s;
}

}  // namespace

extern "C" {

int phx_hessian_blocks_noalloc(int32_t num_nodes, int32_t num_tets, int32_t num_lower_blocks, const int32_t* tets,
                               const double* rest, const uint8_t* model, const double* x, const double* X0,
                               const int32_t* seg_ptr, const int32_t* seg_c, double* blocks, void* stream) {
  if (num_nodes <= 0 || num_tets <= 0 || num_lower_blocks <= 0)
    return fail(PHX_EINVAL, "phx_hessian_blocks_noalloc: sizes must be positive");
  if (num_tets > PHX_NOALLOC_MAX_TETS)
    return fail(PHX_EINVAL, "phx_hessian_blocks_noalloc: " + std::to_string(num_tets) +
                                " tets exceed the fixed scratch of PHX_NOALLOC_MAX_TETS = " +
                                std::to_string(PHX_NOALLOC_MAX_TETS));
  if (!tets || !rest || !x || !X0 || !seg_ptr || !seg_c || !blocks)
    return fail(PHX_EINVAL, "phx_hessian_blocks_noalloc: NULL device pointer");
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_noalloc_elem<<<(num_tets + 127) / 128, 128, 0, s>>>(num_tets, tets, rest, model, x, X0, scratch);
  const int64_t items = 9 * (int64_t)num_lower_blocks;
  k_noalloc_assemble<<<(unsigned)((items + 287) / 288), 288, 0, s>>>(num_lower_blocks, seg_ptr, seg_c, scratch,
                                                                     blocks);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PHX_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
  return PHX_OK;
}

}  // extern "C"
