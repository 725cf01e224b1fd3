// prop_spread.cu -- single propagations, small batches and the Chi3 pump march on a cluster of four CTAs
// with one point per thread (prop_spread.cuh), for grids whose four-points-per-thread cluster form
// would leave schedulers idle or is not built (N = 128 to 1024: M = N/4 threads per CTA); the pump
// march also on eight CTAs for 2048 and 4096 points.
#include <vector>

#include "nlm_launch.h"
#include "prop_spread.cuh"

namespace nlm {

cudaError_t launch_pump_chi3_spread(double2* pumpFreq, double2* pumpTime, const double2* env, const double2* halfP,
                                    const double2* dstepP, const double2* backP, const double2* rel, int nRows, int N,
                                    const double2* tw, cudaStream_t s) {
  // four CTAs up to 1024 points, eight above (M = N / C threads per CTA)
  const int C = N <= 1024 ? 4 : 8;
  int M = N / C;
  if (N % C != 0 || M < 32 || M > kMaxThreads || (M & (M - 1)) != 0) return cudaErrorInvalidValue;
  const void* fn = C == 4 ? (const void*)k_pump_chi3_spread<4> : (const void*)k_pump_chi3_spread<8>;
  // each CTA alone on its SM: its M/32 warps are then the only ones on their schedulers
  size_t smem = 0;
  cudaError_t e = exclusive_smem(fn, (size_t)spread_smem_per_point(C) * M * sizeof(double2), &smem);
  if (e != cudaSuccess) return e;
  if (smem == 0) return cudaErrorInvalidValue;
  void* args[] = {(void*)&pumpFreq, (void*)&pumpTime, (void*)&env, (void*)&halfP, (void*)&dstepP, (void*)&backP,
                  (void*)&rel, (void*)&nRows, (void*)&M, (void*)&tw};
  return launch_clustered(fn, C, M, smem, s, C, args);
}

// key = solver id, R = 1 (one point per thread); cluster of four CTAs of N / 4 threads
void add_kernels_spread(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3, 1, (const void*)k_propagate_spread<FChi3, 4>});
  t.push_back({kKindCluster, kChi2PDC, 1, (const void*)k_propagate_spread<FChi2PDC, 4>});
  t.push_back({kKindCluster, kChi2SFG, 1, (const void*)k_propagate_spread<FChi2SFG, 4>});
  t.push_back({kKindCluster, kChi2AFC, 1, (const void*)k_propagate_spread<FChi2AFC, 4>});
  t.push_back({kKindCluster, kChi2SFGPDC, 1, (const void*)k_propagate_spread<FChi2SFGPDC, 4>});
  t.push_back({kKindCluster, kChi2PDCII, 1, (const void*)k_propagate_spread<FChi2PDCII, 4>});
  t.push_back({kKindCluster, kChi2SFGOPA, 1, (const void*)k_propagate_spread<FChi2SFGOPA, 4>});
  t.push_back({kKindCluster, kChi2SFGXPM, 1, (const void*)k_propagate_spread<FChi2SFGXPM, 4>});
  t.push_back({kKindCluster, kChi2SFGII, 1, (const void*)k_propagate_spread<FChi2SFGII, 4>});
  t.push_back({kKindCluster, kChi2SHG, 1, (const void*)k_propagate_spread<FChi2SHG, 4>});
  t.push_back({kKindCluster, kChi2ASHG, 1, (const void*)k_propagate_spread<FChi2ASHG, 4>});
  t.push_back({kKindCluster, kChi2SHGXPM, 1, (const void*)k_propagate_spread<FChi2SHGXPM, 4>});
  t.push_back({kKindCluster, kChi2SHGOPA, 1, (const void*)k_propagate_spread<FChi2SHGOPA, 4>});
  t.push_back({kKindCluster, kChi2DSFG, 1, (const void*)k_propagate_spread<FChi2DSFG, 4>});
}

}  // namespace nlm
