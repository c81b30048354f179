// pof_linear_filtsmooth_noalloc: the filter + smoother pass without a
// caller-provided workspace, for callers that cannot allocate device memory
// (plugin hosts that only hand out input and output buffers, programs whose
// device memory is owned by another allocator, real-time loops that must
// not call cudaMalloc after start-up).
//
// The scratch memory lives in one file-scope device array of
// POF_NOALLOC_SCRATCH_BYTES, which every GPU that loads libpof holds until
// the process exits.  All calls share it: two calls whose work overlaps on
// the GPU (different streams, or different host threads) race on it, so
// callers must serialize them.  The pass writes every scratch word it reads
// before reading it (it zeroes its own scalar block first), so nothing has
// to be cleared between calls even though the array keeps the previous
// call's contents.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pof.h"

// Device-side scratch shared by every call (host code must not use this
// name as a pointer: on the host it only stands in for the symbol).
static __device__ __align__(256) unsigned char pof_noalloc_scratch[POF_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up once
// per device (the lookup also makes the runtime load the module there).
// The address is kept for the life of the process, so resetting a device
// (cudaDeviceReset) after the first call on it is not supported: the module
// and its array are gone and the kept address is stale.
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return POF_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return POF_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, pof_noalloc_scratch);
    if (e != cudaSuccess || !p) return POF_ERR_CUDA;
    g_ptr[dev] = p;
  }
  *out = g_ptr[dev];
  return POF_OK;
}

}  // namespace

extern "C" int pof_linear_filtsmooth_noalloc(int32_t dtype, int64_t n_steps, int32_t D, int32_t d,
                                             const void* x0_mean, const void* x0_chol, const void* F,
                                             const void* QL, int64_t ft_stride, const void* H, const void* c,
                                             const void* R, int64_t r_stride, void* out_mean, void* out_chol,
                                             double* out_scalars, void* stream) {
  // The argument checks of pof_linear_filtsmooth come first, in its order,
  // so both entry points return the same status for the same bad inputs;
  // then a problem too large for the fixed scratch is refused before
  // touching the GPU.
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (n_steps < 1 || D < 1 || d < 1) return POF_ERR_ARG;
  // (uncompiled shapes with D >= 32 take the dense path, as in pof_linear_filtsmooth)
  if (!pof_shape_supported(D, d) && D < 32) return POF_ERR_SHAPE;
  const size_t need = pof_filtsmooth_workspace_bytes(dtype, n_steps, D, d);
  if (need == 0) return POF_ERR_ARG;
  if (need > (size_t)POF_NOALLOC_SCRATCH_BYTES) return POF_ERR_WORKSPACE;
  void* scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != POF_OK) return rc;
  return pof_linear_filtsmooth(dtype, n_steps, D, d, x0_mean, x0_chol, F, QL, ft_stride, H, c, R, r_stride,
                               out_mean, out_chol, out_scalars, scratch, (size_t)POF_NOALLOC_SCRATCH_BYTES, stream);
}
