// prop_gen_b.cu -- direct-DiffEq kernels for the general plan (FFTPlanH::gen: grids that are not powers of two,
// and power-of-two grids too large for the register plan of a one-CTA kernel) of three two-mode pump-driven solvers.
// R = 8 up to 4096 points, R = 16 up to 8192 (T = ceil(N/R) <= 512 threads).
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_gen_b(std::vector<KernelEntry>& t) {
#define NLM_GEN(S, id, R) t.push_back({kKindDirect, id + kGenKey, R, (const void*)k_propagate_direct<S, R, true>});
  NLM_GEN(FChi2SFG, kChi2SFG, 8)
  NLM_GEN(FChi2SFG, kChi2SFG, 16)
  NLM_GEN(FChi2AFC, kChi2AFC, 8)
  NLM_GEN(FChi2AFC, kChi2AFC, 16)
  NLM_GEN(FChi2SFGPDC, kChi2SFGPDC, 8)
  NLM_GEN(FChi2SFGPDC, kChi2SFGPDC, 16)
#undef NLM_GEN
}

}  // namespace nlm
