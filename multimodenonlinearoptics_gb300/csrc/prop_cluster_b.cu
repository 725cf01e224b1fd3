// prop_cluster_b.cu -- cluster-distributed propagation kernels (nlm_cluster.cuh) of the four-mode
// pump-driven solver and of the fully nonlinear solvers (all but Chi3GNLSE, whose RK4 stages hold
// transforms of their own).
#include <vector>

#include "nlm_cluster.cuh"

namespace nlm {

// key = solver id, R = C (the cluster size)
void add_kernels_cluster_b(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi2SFGII, 4, (const void*)k_propagate_cluster<FChi2SFGII, 4>});
  t.push_back({kKindCluster, kChi2SHG, 4, (const void*)k_propagate_cluster<FChi2SHG, 4>});
  t.push_back({kKindCluster, kChi2ASHG, 4, (const void*)k_propagate_cluster<FChi2ASHG, 4>});
  t.push_back({kKindCluster, kChi2SHGXPM, 4, (const void*)k_propagate_cluster<FChi2SHGXPM, 4>});
  t.push_back({kKindCluster, kChi2SHGOPA, 4, (const void*)k_propagate_cluster<FChi2SHGOPA, 4>});
  t.push_back({kKindCluster, kChi2DSFG, 4, (const void*)k_propagate_cluster<FChi2DSFG, 4>});
}

}  // namespace nlm
