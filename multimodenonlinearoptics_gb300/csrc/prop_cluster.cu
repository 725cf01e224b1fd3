// prop_cluster.cu -- cluster-distributed propagation kernels (nlm_cluster.cuh) of the one- and
// two-mode pump-driven solvers.
#include <vector>

#include "nlm_cluster.cuh"

namespace nlm {

// key = solver id, R = C (the cluster size)
void add_kernels_cluster(std::vector<KernelEntry>& t) {
  t.push_back({kKindCluster, kChi3, 4, (const void*)k_propagate_cluster<FChi3, 4>});
  t.push_back({kKindCluster, kChi2PDC, 4, (const void*)k_propagate_cluster<FChi2PDC, 4>});
  t.push_back({kKindCluster, kChi2SFG, 4, (const void*)k_propagate_cluster<FChi2SFG, 4>});
  t.push_back({kKindCluster, kChi2AFC, 4, (const void*)k_propagate_cluster<FChi2AFC, 4>});
  t.push_back({kKindCluster, kChi2SFGPDC, 4, (const void*)k_propagate_cluster<FChi2SFGPDC, 4>});
  t.push_back({kKindCluster, kChi2PDCII, 4, (const void*)k_propagate_cluster<FChi2PDCII, 4>});
  t.push_back({kKindCluster, kChi2SFGOPA, 4, (const void*)k_propagate_cluster<FChi2SFGOPA, 4>});
  t.push_back({kKindCluster, kChi2SFGXPM, 4, (const void*)k_propagate_cluster<FChi2SFGXPM, 4>});
}

}  // namespace nlm
