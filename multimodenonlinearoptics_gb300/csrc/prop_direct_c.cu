// prop_direct_c.cu -- direct-DiffEq kernels with four points per thread for the one- and two-mode
// solvers.  Launches with fewer propagations than SMs use them so that one propagation has N/4
// threads (four or more warps at N >= 512): the FP64 units of all four schedulers of its SM work on it.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_direct_c(std::vector<KernelEntry>& t) {
  t.push_back({kKindDirect, kChi3, 4, (const void*)k_propagate_direct<FChi3, 4>});
  t.push_back({kKindDirect, kChi2PDC, 4, (const void*)k_propagate_direct<FChi2PDC, 4>});
  t.push_back({kKindDirect, kChi2SFG, 4, (const void*)k_propagate_direct<FChi2SFG, 4>});
  t.push_back({kKindDirect, kChi2AFC, 4, (const void*)k_propagate_direct<FChi2AFC, 4>});
  t.push_back({kKindDirect, kChi2SFGPDC, 4, (const void*)k_propagate_direct<FChi2SFGPDC, 4>});
  t.push_back({kKindDirect, kChi2PDCII, 4, (const void*)k_propagate_direct<FChi2PDCII, 4>});
  t.push_back({kKindDirect, kChi2SFGOPA, 4, (const void*)k_propagate_direct<FChi2SFGOPA, 4>});
  t.push_back({kKindDirect, kChi2SFGXPM, 4, (const void*)k_propagate_direct<FChi2SFGXPM, 4>});
  t.push_back({kKindDirect, kChi2SHG, 4, (const void*)k_propagate_direct<FChi2SHG, 4>});
  t.push_back({kKindDirect, kChi2ASHG, 4, (const void*)k_propagate_direct<FChi2ASHG, 4>});
  t.push_back({kKindDirect, kChi2SHGXPM, 4, (const void*)k_propagate_direct<FChi2SHGXPM, 4>});
}

}  // namespace nlm
