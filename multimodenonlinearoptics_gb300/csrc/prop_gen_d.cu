// prop_gen_d.cu -- direct-DiffEq kernels for the general plan (FFTPlanH::gen: grids that are not powers of two,
// and power-of-two grids too large for the register plan of a one-CTA kernel) of the two-mode fully nonlinear solvers.
// R = 8 up to 4096 points, R = 16 up to 8192 (T = ceil(N/R) <= 512 threads).
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_gen_d(std::vector<KernelEntry>& t) {
#define NLM_GEN(S, id, R) t.push_back({kKindDirect, id + kGenKey, R, (const void*)k_propagate_direct<S, R, true>});
  NLM_GEN(FChi2SHG, kChi2SHG, 8)
  NLM_GEN(FChi2SHG, kChi2SHG, 16)
  NLM_GEN(FChi2ASHG, kChi2ASHG, 8)
  NLM_GEN(FChi2ASHG, kChi2ASHG, 16)
  NLM_GEN(FChi2SHGXPM, kChi2SHGXPM, 8)
  NLM_GEN(FChi2SHGXPM, kChi2SHGXPM, 16)
#undef NLM_GEN
}

}  // namespace nlm
