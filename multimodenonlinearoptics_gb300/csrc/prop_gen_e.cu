// prop_gen_e.cu -- direct-DiffEq kernels for the general plan (FFTPlanH::gen: grids that are not powers of two,
// and power-of-two grids too large for the register plan of a one-CTA kernel) of the four-mode solvers.
// R = 4 up to 2048 points, R = 16 up to 8192 (T = ceil(N/R) <= 512 threads).
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_gen_e(std::vector<KernelEntry>& t) {
#define NLM_GEN(S, id, R) t.push_back({kKindDirect, id + kGenKey, R, (const void*)k_propagate_direct<S, R, true>});
  NLM_GEN(FChi2SFGII, kChi2SFGII, 4)
  NLM_GEN(FChi2SFGII, kChi2SFGII, 16)
  NLM_GEN(FChi2SHGOPA, kChi2SHGOPA, 4)
  NLM_GEN(FChi2SHGOPA, kChi2SHGOPA, 16)
  NLM_GEN(FChi2DSFG, kChi2DSFG, 4)
  NLM_GEN(FChi2DSFG, kChi2DSFG, 16)
#undef NLM_GEN
}

}  // namespace nlm
