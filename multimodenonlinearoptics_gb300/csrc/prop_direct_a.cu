// prop_direct_a.cu -- direct-DiffEq kernels of the single- and two-mode pump-driven solvers.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_direct_a(std::vector<KernelEntry>& t) {
  t.push_back({kKindDirect, kChi3, 8, (const void*)k_propagate_direct<FChi3, 8>});
  t.push_back({kKindDirect, kChi3, 16, (const void*)k_propagate_direct<FChi3, 16>});
  t.push_back({kKindDirect, kChi2PDC, 8, (const void*)k_propagate_direct<FChi2PDC, 8>});
  t.push_back({kKindDirect, kChi2PDC, 16, (const void*)k_propagate_direct<FChi2PDC, 16>});
  t.push_back({kKindDirect, kChi2SFG, 8, (const void*)k_propagate_direct<FChi2SFG, 8>});
  t.push_back({kKindDirect, kChi2AFC, 8, (const void*)k_propagate_direct<FChi2AFC, 8>});
  t.push_back({kKindDirect, kChi2SFGPDC, 8, (const void*)k_propagate_direct<FChi2SFGPDC, 8>});
  t.push_back({kKindDirect, kChi2PDCII, 8, (const void*)k_propagate_direct<FChi2PDCII, 8>});
  t.push_back({kKindDirect, kChi2SFGOPA, 8, (const void*)k_propagate_direct<FChi2SFGOPA, 8>});
  t.push_back({kKindDirect, kChi2SFGXPM, 8, (const void*)k_propagate_direct<FChi2SFGXPM, 8>});
}

}  // namespace nlm
