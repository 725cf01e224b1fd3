// prop_gen_c.cu -- direct-DiffEq kernels for the general plan (FFTPlanH::gen: grids that are not powers of two,
// and power-of-two grids too large for the register plan of a one-CTA kernel) of the other two-mode pump-driven solvers.
// R = 8 up to 4096 points, R = 16 up to 8192 (T = ceil(N/R) <= 512 threads).
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_gen_c(std::vector<KernelEntry>& t) {
#define NLM_GEN(S, id, R) t.push_back({kKindDirect, id + kGenKey, R, (const void*)k_propagate_direct<S, R, true>});
  NLM_GEN(FChi2PDCII, kChi2PDCII, 8)
  NLM_GEN(FChi2PDCII, kChi2PDCII, 16)
  NLM_GEN(FChi2SFGOPA, kChi2SFGOPA, 8)
  NLM_GEN(FChi2SFGOPA, kChi2SFGOPA, 16)
  NLM_GEN(FChi2SFGXPM, kChi2SFGXPM, 8)
  NLM_GEN(FChi2SFGXPM, kChi2SFGXPM, 16)
#undef NLM_GEN
}

}  // namespace nlm
