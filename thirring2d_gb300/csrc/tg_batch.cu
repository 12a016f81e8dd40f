// tg_batch.cu -- the batched-chain kernel's instances with one thread block
// per chain, the instance table the autotuner chooses from, and dispatch
// (cluster instances: tg_batch_cluster.cu).
#include <algorithm>

#include "tg_batch_impl.cuh"

namespace tg {

template <int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_batch_trajectory(const BatchChain* __restrict__ chains,
                                                               const int* __restrict__ order, int n,
                                                               BatchFields F, BatchTraj P, ChainResult* results,
                                                               unsigned long long* queue) {
  batch_trajectory_body<BS, MINB, BlockTeam>(chains, order, n, F, P, results, queue);
}

// The kernel instances the autotuner chooses from: (threads per block,
// minimum resident blocks per SM).  More blocks per SM cap the registers (64 at
// 2048 resident threads, with spills in the column march); fewer leave room
// for the march's registers (up to 255 at 256 threads and one block).
// The cluster instances split each chain over 2 or 4 SMs; their variants with
// solo_sites hand the chains of up to 64^2 or 96^2 sites (the end of the
// largest-first queue) to single blocks, which no longer wait on cluster
// barriers.
const BatchCfg kBatchCfgs[kBatchNumCfgs] = {
    {128, 8, 1, 0},    {256, 4, 1, 0},    {256, 2, 1, 0},    {256, 1, 1, 0},    {384, 1, 1, 0},
    {512, 1, 1, 0},    {512, 1, 2, 0},    {512, 1, 4, 0},    {256, 1, 4, 0},    {512, 1, 2, 4096},
    {512, 1, 2, 9216}, {512, 1, 4, 4096}, {512, 1, 4, 9216}, {256, 1, 4, 4096}, {256, 1, 4, 9216},
    {512, 1, 4, 4096, 1}};

// the cluster kernel of instance cfg (see batch_cluster_max)
static int cluster_kernel_of(int cfg) {
  const BatchCfg& c = kBatchCfgs[cfg];
  if (c.pairs) return 3;
  return c.cluster == 2 ? 0 : (c.block == 512 ? 1 : 2);
}

template <int BS, int MINB> const void* batch_kernel() { return (const void*)k_batch_trajectory<BS, MINB>; }

static const void* batch_kernel_of(int cfg) {
  switch (cfg) {
    case 0: return batch_kernel<128, 8>();
    case 1: return batch_kernel<256, 4>();
    case 2: return batch_kernel<256, 2>();
    case 3: return batch_kernel<256, 1>();
    case 4: return batch_kernel<384, 1>();
    default: return batch_kernel<512, 1>();
  }
}

static void launch_blocks(cudaStream_t s, int cfg, int grid, const BatchChain* chains, const int* order, int n,
                          const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue) {
  switch (cfg) {
    case 0: k_batch_trajectory<128, 8><<<grid, 128, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 1: k_batch_trajectory<256, 4><<<grid, 256, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 2: k_batch_trajectory<256, 2><<<grid, 256, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 3: k_batch_trajectory<256, 1><<<grid, 256, 0, s>>>(chains, order, n, F, P, results, queue); break;
    case 4: k_batch_trajectory<384, 1><<<grid, 384, 0, s>>>(chains, order, n, F, P, results, queue); break;
    default: k_batch_trajectory<512, 1><<<grid, 512, 0, s>>>(chains, order, n, F, P, results, queue); break;
  }
}

int batch_teams(int cfg, int sms) {
  if (kBatchCfgs[cfg].cluster > 1) return batch_cluster_max(cluster_kernel_of(cfg));
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_kernel_of(cfg), kBatchCfgs[cfg].block, 0) !=
      cudaSuccess)
    return 0;
  return nb * sms;
}

int batch_filler_blocks(int cfg, int sms) {
  const BatchCfg& c = kBatchCfgs[cfg];
  if (c.cluster <= 1 || c.solo_sites <= 0) return 0;
  const int clusters = batch_cluster_max(cluster_kernel_of(cfg));
  return std::max(0, sms - clusters * c.cluster);
}

void batch_filler_launch(cudaStream_t s, int cfg, int blocks, const BatchChain* chains, const int* order, int n,
                         const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue) {
  BatchTraj f = P;
  f.from_back = 1;
  // the one-block instance of the cluster kernel's block size: its solo chains
  // run the same code, so a chain's result does not depend on which block ran it
  if (kBatchCfgs[cfg].block == 512)
    k_batch_trajectory<512, 1><<<blocks, 512, 0, s>>>(chains, order, n, F, f, results, queue);
  else
    k_batch_trajectory<256, 1><<<blocks, 256, 0, s>>>(chains, order, n, F, f, results, queue);
}

void batch_trajectory(cudaStream_t s, int cfg, int sms, const BatchChain* chains, const int* order, int n,
                      const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue) {
  const int teams = std::min(n, std::max(1, batch_teams(cfg, sms)));
  if (kBatchCfgs[cfg].cluster > 1)
    batch_cluster_launch(s, cluster_kernel_of(cfg), teams, chains, order, n, F, P, results, queue);
  else launch_blocks(s, cfg, teams, chains, order, n, F, P, results, queue);
}

}  // namespace tg
