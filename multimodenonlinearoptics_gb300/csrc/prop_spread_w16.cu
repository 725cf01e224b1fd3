// prop_spread_w16.cu -- the one-point-per-thread cluster kernels (prop_spread.cuh) on sixteen CTAs, a
// non-portable cluster size: 2048- and 4096-point propagations with N/16 points per CTA, for the
// marches that set a ragged batch's makespan (and cluster mode 3).  Multi-mode solvers only in the form
// that transforms their modes together (the form with one mode after another would spill registers),
// where its buffers fit in shared memory (spread_smem_per_point_k: 2048 points).
#include <vector>

#include "prop_spread.cuh"

namespace nlm {

// kind kKindCluster (single-mode solvers) / kKindSpreadFused (multi-mode), key = solver id +
// kSpreadW16Key, R = 1 (one point per thread)
void add_kernels_spread_w16(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3 + kSpreadW16Key, 1, (const void*)k_propagate_spread<FChi3, 16>});
  t.push_back({kKindCluster, kChi2PDC + kSpreadW16Key, 1, (const void*)k_propagate_spread<FChi2PDC, 16>});
#define NLM_W16_FUSED(S, id) \
  t.push_back({kKindSpreadFused, id + kSpreadW16Key, 1, (const void*)k_propagate_spread<S, 16, S::kM>});
  NLM_W16_FUSED(FChi2SFG, kChi2SFG)
  NLM_W16_FUSED(FChi2AFC, kChi2AFC)
  NLM_W16_FUSED(FChi2SFGPDC, kChi2SFGPDC)
  NLM_W16_FUSED(FChi2PDCII, kChi2PDCII)
  NLM_W16_FUSED(FChi2SFGOPA, kChi2SFGOPA)
  NLM_W16_FUSED(FChi2SFGXPM, kChi2SFGXPM)
  NLM_W16_FUSED(FChi2SFGII, kChi2SFGII)
  NLM_W16_FUSED(FChi2SHG, kChi2SHG)
  NLM_W16_FUSED(FChi2ASHG, kChi2ASHG)
  NLM_W16_FUSED(FChi2SHGXPM, kChi2SHGXPM)
  NLM_W16_FUSED(FChi2SHGOPA, kChi2SHGOPA)
  NLM_W16_FUSED(FChi2DSFG, kChi2DSFG)
#undef NLM_W16_FUSED
}

}  // namespace nlm
