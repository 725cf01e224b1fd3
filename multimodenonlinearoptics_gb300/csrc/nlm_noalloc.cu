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
//    the library holds it until the process exits.  A grid needs 2 N complex values per resident
//    propagation; grids for which one CTA's propagations do not fit are rejected with
//    NLM_ERR_INVALID_ARGUMENT.  Fewer resident propagations only means more rounds of the
//    persistent kernel, so any number of rows is accepted.
//  * Every call uses the same array and leaves its contents behind.  The kernel writes each slot
//    (state from the input, accumulator at the first RK4 stage) before reading it, so nothing has
//    to be cleared between calls.  Calls whose kernels overlap on the GPU (for example on two
//    streams) race on the array: serialise them.
//  * The first call on a device looks up the array's device address (cudaGetSymbolAddress, with that
//    device current) and caches it; make that first call before any stream capture.
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

// Device address of g_noalloc_scratch on each device, looked up once per device.
static cudaError_t scratch_address(double2** ptr) {
  static std::mutex mu;
  static double2* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
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
  cudaError_t e = nlm::scratch_address(&scratch);
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
