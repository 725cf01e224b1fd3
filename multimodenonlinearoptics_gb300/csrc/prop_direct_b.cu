// prop_direct_b.cu -- direct-DiffEq kernels of the four-mode and fully nonlinear solvers.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_direct_b(std::vector<KernelEntry>& t) {
  t.push_back({kKindDirect, kChi2SFGII, 4, (const void*)k_propagate_direct<FChi2SFGII, 4>});
  t.push_back({kKindDirect, kChi2SHG, 8, (const void*)k_propagate_direct<FChi2SHG, 8>});
  t.push_back({kKindDirect, kChi2ASHG, 8, (const void*)k_propagate_direct<FChi2ASHG, 8>});
  t.push_back({kKindDirect, kChi2SHGXPM, 8, (const void*)k_propagate_direct<FChi2SHGXPM, 8>});
  t.push_back({kKindDirect, kChi2SHGOPA, 4, (const void*)k_propagate_direct<FChi2SHGOPA, 4>});
  t.push_back({kKindDirect, kChi2DSFG, 4, (const void*)k_propagate_direct<FChi2DSFG, 4>});
}

}  // namespace nlm
