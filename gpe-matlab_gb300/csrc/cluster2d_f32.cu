// The persistent cluster kernel of small 2D grids, float instantiation.
#include "cluster2d.cuh"

namespace gpe {
template <>
cudaError_t launch_cluster2d<float>(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s) {
  return launch_cluster2d_impl<float>(a, nclusters, cs, smem, s);
}
template <>
int cluster2d_max_clusters<float>(int cs, size_t smem) {
  return cluster2d_max_clusters_impl<float>(cs, smem);
}
}  // namespace gpe
