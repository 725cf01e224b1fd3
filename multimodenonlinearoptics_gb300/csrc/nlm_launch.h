// nlm_launch.h -- host helpers for the thread-block-cluster launches of the engine.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

namespace nlm {

// Dynamic shared memory for a kernel whose CTAs each take a whole SM: at least `need` bytes and more
// than half of what one CTA may have, so that no second CTA fits beside it (a latency-bound march
// then shares its SM's FP64 units with nothing else).  Raises the kernel's dynamic shared-memory
// limit accordingly.  *smem = 0 when `need` does not fit; *attr (optional) gets the kernel's
// attributes.
inline cudaError_t exclusive_smem(const void* fn, size_t need, size_t* smem, cudaFuncAttributes* attr = nullptr) {
  *smem = 0;
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return e;
  if (attr) *attr = fa;
  const int dynMax = optin - (int)fa.sharedSizeBytes;
  if ((long long)need > (long long)dynMax) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dynMax);
  if (e != cudaSuccess) return e;
  *smem = std::max<size_t>(need, (size_t)dynMax / 2 + 1024);
  return cudaSuccess;
}

// A launch configuration with a one-dimensional cluster of `clusterSize` CTAs; `attr` is the
// storage of its one launch attribute.
inline cudaLaunchConfig_t cluster_config(int grid, int block, size_t smem, cudaStream_t s, int clusterSize,
                                         cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr->id = cudaLaunchAttributeClusterDimension;
  attr->val.clusterDim.x = (unsigned)clusterSize;
  attr->val.clusterDim.y = 1;
  attr->val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

inline cudaError_t launch_clustered(const void* fn, int grid, int block, size_t smem, cudaStream_t s, int clusterSize,
                                    void** args) {
  cudaLaunchAttribute attr;
  cudaLaunchConfig_t cfg = cluster_config(grid, block, smem, s, clusterSize, &attr);
  return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace nlm
