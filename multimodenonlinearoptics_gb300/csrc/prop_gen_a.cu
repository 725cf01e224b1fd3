// prop_gen_a.cu -- direct-DiffEq kernels for the general plan (FFTPlanH::gen: grids that are not powers of two,
// and power-of-two grids too large for the register plan of a one-CTA kernel) of the single-mode solvers.
// R = 8 up to 4096 points, R = 16 up to 8192 (T = ceil(N/R) <= 512 threads).
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_gen_a(std::vector<KernelEntry>& t) {
#define NLM_GEN(S, id, R) t.push_back({kKindDirect, id + kGenKey, R, (const void*)k_propagate_direct<S, R, true>});
  NLM_GEN(FChi3, kChi3, 8)
  NLM_GEN(FChi3, kChi3, 16)
  NLM_GEN(FChi2PDC, kChi2PDC, 8)
  NLM_GEN(FChi2PDC, kChi2PDC, 16)
#undef NLM_GEN
}

}  // namespace nlm
