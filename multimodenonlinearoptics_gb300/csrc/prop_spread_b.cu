// prop_spread_b.cu -- the one-point-per-thread cluster kernels (prop_spread.cuh) on eight CTAs, for
// 2048- and 4096-point grids (M = N/8 threads per CTA): twice the SMs of the four-points-per-thread
// cluster form.  Used for full-grid propagations and the media of ragged batches, whose launches no
// reverse sweep pairs with.
#include <vector>

#include "prop_spread.cuh"

namespace nlm {

// key = solver id + kSpreadWideKey, R = 1 (one point per thread); cluster of eight CTAs
void add_kernels_spread_b(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3 + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi3, 8>});
  t.push_back({kKindCluster, kChi2PDC + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2PDC, 8>});
  t.push_back({kKindCluster, kChi2SFG + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SFG, 8>});
  t.push_back({kKindCluster, kChi2AFC + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2AFC, 8>});
  t.push_back({kKindCluster, kChi2SFGPDC + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SFGPDC, 8>});
  t.push_back({kKindCluster, kChi2PDCII + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2PDCII, 8>});
  t.push_back({kKindCluster, kChi2SFGOPA + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SFGOPA, 8>});
  t.push_back({kKindCluster, kChi2SFGXPM + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SFGXPM, 8>});
  t.push_back({kKindCluster, kChi2SFGII + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SFGII, 8>});
  t.push_back({kKindCluster, kChi2SHG + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SHG, 8>});
  t.push_back({kKindCluster, kChi2ASHG + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2ASHG, 8>});
  t.push_back({kKindCluster, kChi2SHGXPM + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SHGXPM, 8>});
  t.push_back({kKindCluster, kChi2SHGOPA + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2SHGOPA, 8>});
  t.push_back({kKindCluster, kChi2DSFG + kSpreadWideKey, 1, (const void*)k_propagate_spread<FChi2DSFG, 8>});
}

}  // namespace nlm
