// tg_batch.h -- structures and launch interface of the batched-chain kernel
// (tg_batch.cu), shared with the C ABI in tg_capi.cu.
#pragma once

#include "tg_internal.cuh"

namespace tg {

// One chain: geometry, couplings, seed, and where its sites start in the
// packed field arrays (chains are concatenated site-major).
struct BatchChain {
  Geo geo;
  double m, g, mu;
  int bc_t, bc_x;
  unsigned long long seed;
  long long off;
};

// Packed per-site fields of all chains.
struct BatchFields {
  double2 *A, *An, *mom, *phi, *noise, *x, *Mx, *tmp, *Wt, *Wx, *r64, *p64, *p64b, *Mp64;
  float2 *Wt32, *Wx32, *xs, *rs, *ps, *ps2, *Mps;  // p64/p64b, ps/ps2: CG directions of alternate iterations
};

struct BatchCg {
  double rel_tol, abs_tol2;
  int maxiter, precision, ru_interval;
};

struct BatchTraj {
  int nsteps;
  double tau;
  int stochastic_term;
  BatchCg cg;
  // cluster instances: from this queue position on, every block of a cluster
  // runs chains of its own (n: never)
  int solo_from;
  // 1 for the filler blocks beside a cluster launch: they take chains from the
  // back of the queue, at or after solo_from only
  int from_back;
  // 4-block cluster instances with pairs: queue positions [solo_from, pair_end)
  // run on two blocks each (PairTeam), later ones on one (pair_end = solo_from:
  // no pairs)
  int pair_end;
};

// Per-chain outcome of a trajectory; `traj` is the chain's Philox trajectory
// counter (read at the start, incremented at the end).
struct ChainResult {
  double dH, Sg0, Spf0, Smd0, Smom0, Sg1, Spf1, Smd1, Smom1, u;
  int accepted, status, cg_iterations, cg_max_iterations, reliable_updates, solves;
  unsigned long long traj;
};

// kernel instances of the batched trajectory: threads per block, min blocks per
// SM, blocks per chain (1: one block per chain; > 1: a thread-block cluster),
// and for clusters the chain size (sites) at or below which the cluster's
// blocks split up and run one chain each (0: never).  `pairs` (4-block
// clusters): only the chains whose estimated cost exceeds twice an SM's share
// of the batch run on four blocks; the rest of the queue up to the first small
// chain runs on pairs of blocks (PairTeam), the queue staying largest-first.
struct BatchCfg {
  int block, minb, cluster, solo_sites, pairs;
};
constexpr int kBatchNumCfgs = 16;
extern const BatchCfg kBatchCfgs[kBatchNumCfgs];

// The work queue is one 64-bit word (0 at launch): the low half counts the
// chains taken from its front (teams, largest estimated cost first), the high
// half those taken from its back (filler blocks, the cheapest chains).
//
// Launches instance cfg over n chains with as many teams as can be resident.
void batch_trajectory(cudaStream_t s, int cfg, int sms, const BatchChain* chains, const int* order, int n,
                      const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue);
// Cluster instances with solo chains leave SMs that hold no whole cluster idle
// (152 SMs take 36 clusters of 4): one-block teams of the same block size run
// there, concurrently on stream s, taking solo chains from the back of the
// queue.  batch_filler_blocks gives their number (0: none for this instance).
int batch_filler_blocks(int cfg, int sms);
void batch_filler_launch(cudaStream_t s, int cfg, int blocks, const BatchChain* chains, const int* order, int n,
                         const BatchFields& F, const BatchTraj& P, ChainResult* results, unsigned long long* queue);
// teams (blocks or clusters) of instance cfg that can be resident at once (0: cannot launch)
int batch_teams(int cfg, int sms);
// the tuned instance as reported to callers: block * 100 + 10 * cluster (if > 1)
// + min blocks per SM, + 100000 * (solo_sites / 1024), + 1000000 with pairs
inline int batch_cfg_id(const BatchCfg& c) {
  return c.block * 100 + (c.cluster > 1 ? 10 * c.cluster : 0) + c.minb + 100000 * (c.solo_sites / 1024) +
         1000000 * c.pairs;
}

// tg_batch_cluster.cu: instance `which` (0: 512 x 2 blocks, 1: 512 x 4, 2: 256 x 4,
// 3: 512 x 4 with pairs)
int batch_cluster_max(int which);
void batch_cluster_launch(cudaStream_t s, int which, int clusters, const BatchChain* chains, const int* order, int n,
                          const BatchFields& F, const BatchTraj& P, ChainResult* results,
                          unsigned long long* queue);

}  // namespace tg
