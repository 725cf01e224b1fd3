// prop_spread_fused.cu -- the one-point-per-thread cluster kernels (prop_spread.cuh) of the multi-mode
// solvers with all modes in each transform together: one stage barrier and one cluster barrier per
// transform for every mode instead of one set per mode, and the modes' independent arithmetic in flight
// together on each thread.  Four CTAs (128 to 1024 points) and eight (2048 and 4096 points, where the
// buffers fit: spread_smem_per_point_k).
#include <vector>

#include "prop_spread.cuh"

namespace nlm {

// kind kKindSpreadFused, keys as the unfused kernels: solver id (four CTAs), + kSpreadWideKey (eight)
void add_kernels_spread_fused(std::vector<KernelEntry>& t) {
#define NLM_FUSED(S, id)                                                                                   \
  t.push_back({kKindSpreadFused, id, 1, (const void*)k_propagate_spread<S, 4, S::kM>});                  \
  t.push_back({kKindSpreadFused, id + kSpreadWideKey, 1, (const void*)k_propagate_spread<S, 8, S::kM>});
  NLM_FUSED(FChi2SFG, kChi2SFG)
  NLM_FUSED(FChi2AFC, kChi2AFC)
  NLM_FUSED(FChi2SFGPDC, kChi2SFGPDC)
  NLM_FUSED(FChi2PDCII, kChi2PDCII)
  NLM_FUSED(FChi2SFGOPA, kChi2SFGOPA)
  NLM_FUSED(FChi2SFGXPM, kChi2SFGXPM)
  NLM_FUSED(FChi2SFGII, kChi2SFGII)
  NLM_FUSED(FChi2SHG, kChi2SHG)
  NLM_FUSED(FChi2ASHG, kChi2ASHG)
  NLM_FUSED(FChi2SHGXPM, kChi2SHGXPM)
  NLM_FUSED(FChi2SHGOPA, kChi2SHGOPA)
  NLM_FUSED(FChi2DSFG, kChi2DSFG)
#undef NLM_FUSED
}

}  // namespace nlm
