// nlm_noalloc.cu -- allocation-free variant of the Chi3GNLSE batch propagation.
//
// Who needs it: callers that may not allocate device memory at the point where they propagate --
// code whose device memory is owned by another allocator with a fixed budget (a framework's
// caching pool), or latency-critical loops in which a cudaMalloc/cudaFree (which can synchronise the
// device) is not acceptable.  The ordinary batch entry point allocates its scratch (two N-point
// complex slots per resident propagation, for the field state and the RK4 accumulator) on demand;
// this variant takes that scratch from one file-scope device array instead.
//
// Limits and contract:
//  * The scratch array holds kNoAllocScratchElems complex values (16 MiB).  Every GPU that loads
//    the library holds it until the process exits.  Each resident propagation takes a slot of 2 N
//    complex values, so the array bounds how many CTAs of the persistent kernel run at once (at
//    N = 4096, 128 CTAs, fewer than the SMs of a GB300); fewer resident propagations only means more
//    rounds of the grid, so any number of rows is accepted.  What limits the grid size is shared
//    memory: only grids the one-CTA Chi3GNLSE kernel takes (power of two, 8 to 4096 points) are
//    accepted, others are rejected with NLM_ERR_UNSUPPORTED.
//  * Every call uses the same array and leaves its contents behind.  The kernel writes each slot
//    (state from the input, accumulator at the first RK4 stage) before reading it, so nothing has
//    to be cleared between calls.  Calls whose kernels overlap on the GPU (for example on two
//    streams) race on the array: serialise them.
//  * The medium's tables live on the device that was current when it first ran on the GPU; a call
//    made with another device current is rejected.
//  * The array's device address is looked up (cudaGetSymbolAddress, with the device current) on the
//    first call on a device and again on every call made outside stream capture, so a context
//    recreated after cudaDeviceReset gets the new address; a call made during capture uses the
//    address of the last call made outside it.  Make the first call on a device before any capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/nlm_capi.h"
#include "nlm_kernels.h"

namespace nlm {

constexpr size_t kNoAllocScratchElems = size_t(1) << 20;   // 16 MiB of double2
static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocScratchElems];

nlm_status prepare_gnlse_noalloc(nlm_medium* h, const void* in, size_t rows, int inTime, void* out,
                                 size_t scratchElems, PropArgs* args, int* grid, int* block, size_t* smem,
                                 const void** fn, cudaStream_t* stream);
void set_error_message(const std::string& msg);

// Device address of g_noalloc_scratch on the current device: looked up on the first call on a
// device and on every call outside stream capture (the lookup may load the module, which capture
// does not allow); during capture the last address found on that device.
static cudaError_t scratch_address(cudaStream_t stream, double2** ptr) {
  static std::mutex mu;
  static double2* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev] || cap == cudaStreamCaptureStatusNone) {
    if (cap != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    addr[dev] = static_cast<double2*>(p);
  }
  *ptr = addr[dev];
  return cudaSuccess;
}

}  // namespace nlm

extern "C" nlm_status nlm_batch_gnlse_noalloc(nlm_medium* medium, const void* inputs_dev, size_t rows,
                                              int in_time_domain, void* out_dev, void* cuda_stream) {
  nlm::PropArgs a;
  int grid = 0, block = 0;
  size_t smem = 0;
  const void* fn = nullptr;
  cudaStream_t stream = nullptr;
  nlm_status st = nlm::prepare_gnlse_noalloc(medium, inputs_dev, rows, in_time_domain, out_dev,
                                             nlm::kNoAllocScratchElems, &a, &grid, &block, &smem, &fn, &stream);
  if (st != NLM_OK) return st;
  stream = static_cast<cudaStream_t>(cuda_stream);   // the caller's stream; NULL is the legacy default stream
  double2* scratch = nullptr;
  cudaError_t e = nlm::scratch_address(stream, &scratch);
  if (e == cudaSuccess) {
    void* kargs[] = {(void*)&a, (void*)&scratch};
    e = cudaLaunchKernel(fn, dim3(grid), dim3(block), kargs, smem, stream);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    nlm::set_error_message(std::string("allocation-free GNLSE batch: ") + cudaGetErrorString(e));
    return NLM_ERR_CUDA;
  }
  return NLM_OK;
}
