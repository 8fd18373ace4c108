// The persistent cluster kernel of small 2D grids, double instantiation.
#include "cluster2d.cuh"

namespace gpe {
template <>
cudaError_t launch_cluster2d<double>(const C2Args& a, int nclusters, int cs, size_t smem, cudaStream_t s) {
  return launch_cluster2d_impl<double>(a, nclusters, cs, smem, s);
}
template <>
int cluster2d_max_clusters<double>(int cs, size_t smem) {
  return cluster2d_max_clusters_impl<double>(cs, smem);
}
}  // namespace gpe
