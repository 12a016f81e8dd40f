// tg_batch_cluster.cu -- the batched-chain kernel's instances with one
// thread-block cluster per chain: the chain's rows are split over the CL
// blocks of the cluster (on CL SMs), and its sums go through distributed
// shared memory (ClusterTeam in tg_batch_impl.cuh).  A large chain's operator
// passes and FP64 work then run on CL SMs instead of one.
#include "tg_batch_impl.cuh"

namespace tg {

template <int BS, int CL, bool PAIRS = false>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(BS, 1)
    k_batch_cluster(const BatchChain* __restrict__ chains, const int* __restrict__ order, int n, BatchFields F,
                    BatchTraj P, ChainResult* results, unsigned long long* queue) {
  batch_trajectory_body<BS, 1, ClusterTeam<CL>, PAIRS>(chains, order, n, F, P, results, queue);
}

template <int BS, int CL, bool PAIRS = false> int max_clusters_of() {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(BS);
  cfg.dynamicSmemBytes = 0;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch_cluster<BS, CL, PAIRS>, &cfg) != cudaSuccess) {
    cudaGetLastError();  // clear it: the instance is just not offered
    return 0;
  }
  return n;
}

int batch_cluster_max(int which) {
  switch (which) {
    case 0: return max_clusters_of<512, 2>();
    case 1: return max_clusters_of<512, 4>();
    case 3: return max_clusters_of<512, 4, true>();
    default: return max_clusters_of<256, 4>();
  }
}

void batch_cluster_launch(cudaStream_t s, int which, int clusters, const BatchChain* chains, const int* order, int n,
                          const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue) {
  switch (which) {
    case 0: k_batch_cluster<512, 2><<<clusters * 2, 512, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 1: k_batch_cluster<512, 4><<<clusters * 4, 512, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 3:
      k_batch_cluster<512, 4, true><<<clusters * 4, 512, 0, s>>>(chains, order, n, F, P, results, queue);
      break;
    default: k_batch_cluster<256, 4><<<clusters * 4, 256, 0, s>>>(chains, order, n, F, P, results, queue); break;
  }
}

}  // namespace tg
