// prop_linear.cu -- instantiations of the linear-propagator kernels and of the propagator build.
#include <vector>

#include "nlm_propagate.cuh"

namespace nlm {

void add_kernels_linear(std::vector<KernelEntry>& t) {
  t.push_back({kKindLinear, 1, 8, (const void*)k_propagate_linear<1, 8>});
  t.push_back({kKindLinear, 1, 16, (const void*)k_propagate_linear<1, 16>});
  // autotuner candidates: 128-thread CTAs with 5 or 6 resident per SM (96 / 80 registers)
  t.push_back({kKindLinear, 1, 8, (const void*)k_propagate_linear_occ<1, 8, 5>});
  t.push_back({kKindLinear, 1, 8, (const void*)k_propagate_linear_occ<1, 8, 6>});
  t.push_back({kKindLinear, 2, 8, (const void*)k_propagate_linear<2, 8>});
  t.push_back({kKindLinear, 4, 4, (const void*)k_propagate_linear<4, 4>});
  // latency-bound launches (fewer propagations than SMs): N/4 threads, all four schedulers of the SM
  t.push_back({kKindLinear, 1, 4, (const void*)k_propagate_linear<1, 4>});
  t.push_back({kKindLinear, 2, 4, (const void*)k_propagate_linear<2, 4>});
  // key + kGenKey: grids that are not powers of two (general plan)
  t.push_back({kKindLinear, 1 + kGenKey, 8, (const void*)k_propagate_linear<1, 8, false, true>});
  t.push_back({kKindLinear, 1 + kGenKey, 16, (const void*)k_propagate_linear<1, 16, false, true>});
  t.push_back({kKindLinear, 2 + kGenKey, 8, (const void*)k_propagate_linear<2, 8, false, true>});
  t.push_back({kKindLinear, 4 + kGenKey, 4, (const void*)k_propagate_linear<4, 4, false, true>});
  // key + 100: the adjoint's checkpointed forwards
  t.push_back({kKindLinear, 101, 4, (const void*)k_propagate_linear<1, 4, true>});
  t.push_back({kKindLinear, 101, 8, (const void*)k_propagate_linear<1, 8, true>});
  t.push_back({kKindLinear, 101, 16, (const void*)k_propagate_linear<1, 16, true>});
  // linear (pump-driven) solvers: their RK4 step is real-linear in the signal
  t.push_back({kKindBuildProp, kChi3, 0, (const void*)k_build_propagator<FChi3>});
  t.push_back({kKindBuildProp, kChi2PDC, 0, (const void*)k_build_propagator<FChi2PDC>});
  t.push_back({kKindBuildProp, kChi2SFG, 0, (const void*)k_build_propagator<FChi2SFG>});
  t.push_back({kKindBuildProp, kChi2AFC, 0, (const void*)k_build_propagator<FChi2AFC>});
  t.push_back({kKindBuildProp, kChi2SFGPDC, 0, (const void*)k_build_propagator<FChi2SFGPDC>});
  t.push_back({kKindBuildProp, kChi2SFGII, 0, (const void*)k_build_propagator<FChi2SFGII>});
  t.push_back({kKindBuildProp, kChi2PDCII, 0, (const void*)k_build_propagator<FChi2PDCII>});
  t.push_back({kKindBuildProp, kChi2SFGOPA, 0, (const void*)k_build_propagator<FChi2SFGOPA>});
  t.push_back({kKindBuildProp, kChi2SFGXPM, 0, (const void*)k_build_propagator<FChi2SFGXPM>});
}

}  // namespace nlm
