// tg_batch_impl.cuh -- many independent HMC chains of different lattice sizes,
// masses and couplings in one persistent kernel launch per trajectory.  The
// kernel template lives here; tg_batch.cu instantiates it for one thread block
// per chain, tg_batch_cluster.cu for one thread-block cluster per chain.
//
// Each team (a thread block, or a cluster of blocks on several SMs) takes chains
// from a work queue (largest estimated cost first) and runs a chain's whole
// trajectory team-synchronously: heatbath,
// nsteps leapfrog steps with a CG solve each, forces, Hamiltonian sums,
// accept/reject (hmc.c:671-746).  CG iterations cost block barriers instead of
// kernel launches, so lattices from 16^2 to 128^2 run at full occupancy, and a
// chain's convergence never waits for another chain's.  Random fields come
// from the same Philox streams, keyed by the chain's seed and trajectory
// counter, as the single-lattice path, and the arithmetic uses the same
// device functions (tg_device.cuh), so a chain reproduces a single-lattice
// trajectory with the same seed to rounding.
#pragma once

#include <cooperative_groups.h>
#include <math.h>

#include "tg_batch.h"
#include "tg_stencil.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Block-wide primitives (all threads of the block call them)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Shared scratch of the team sums: the warps' partials, the block's total (read
// by the other blocks of a cluster) and the result of the step that follows a
// sum.
struct TeamScratch {
  double part[32];
  double total[2];  // a cluster's block totals alternate between two slots
  double out[4];
  int phase;        // the slot of the next sum (thread 0 only)
};
__device__ __forceinline__ TeamScratch& team_scratch() {
  __shared__ TeamScratch sc;
  return sc;
}

__device__ __forceinline__ float warp_allsum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// The block's total of the threads' partials (fixed butterfly order), in warp
// 0.  FP32 partials are added in FP32 within a warp (their own rounding is
// FP32's already) and in FP64 from the warps' totals on.
template <typename P> __device__ __forceinline__ double block_total_warp0(P v, TeamScratch& sc) {
  v = warp_allsum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) sc.part[w] = (double)v;
  __syncthreads();  // also publishes every global write made before the call
  return w == 0 ? warp_allsum(lane < nw ? sc.part[lane] : 0.0) : 0.0;
}

// A team runs one chain.  It gives the chain-wide loop over sites, barrier and
// sum; every thread of the team sees the same sums (fixed order), so all make
// the same decisions and the team's control flow stays uniform.
//
// sum_then(v, f): the team's total of the threads' partials v, handed to f,
// which runs once per block (thread 0); every thread gets f's result (a small
// trivially copyable struct).  Scalars derived from a sum -- CG step lengths,
// the stopping tests -- are computed there once instead of in every thread:
// the FP64 pipe retires two operations per SM per clock, and one double
// division is about ten of them.
struct BlockTeam {  // one thread block
  __device__ static int rank() { return 0; }
  __device__ static int nblocks() { return 1; }
  __device__ static void sync() { __syncthreads(); }
  template <typename P, class F> __device__ static auto sum_then(P v, F f) -> decltype(f(0.0)) {
    using S = decltype(f(0.0));
    static_assert(sizeof(S) <= sizeof(TeamScratch::out), "sum_then result too large");
    TeamScratch& sc = team_scratch();
    const double t = block_total_warp0(v, sc);
    if (threadIdx.x == 0) *reinterpret_cast<S*>(sc.out) = f(t);
    __syncthreads();
    return *reinterpret_cast<const S*>(sc.out);
  }
  __device__ static double sum(double v) { return sum_then(v, [](double t) { return t; }); }
  __device__ static void init() {}
  static constexpr bool kCluster = false;
  // the queue ticket thread 0 of rank 0 wrote to `next`
  __device__ static int broadcast(const int* next) {
    __syncthreads();
    return *next;
  }
};

// CL thread blocks of one cluster, on CL SMs.  The cluster barrier orders
// the blocks' global and shared memory accesses; sums combine the blocks'
// totals through distributed shared memory, in the same order in every block,
// so the blocks stay in lockstep.
template <int CL> struct ClusterTeam {
  __device__ static int rank() { return (int)cooperative_groups::this_cluster().block_rank(); }
  __device__ static int nblocks() { return CL; }
  __device__ static void sync() { cooperative_groups::this_cluster().sync(); }
  template <typename P, class F> __device__ static auto sum_then(P v, F f) -> decltype(f(0.0)) {
    using S = decltype(f(0.0));
    static_assert(sizeof(S) <= sizeof(TeamScratch::out), "sum_then result too large");
    TeamScratch& sc = team_scratch();
    const double b = block_total_warp0(v, sc);
    int ph = 0;
    if (threadIdx.x == 0) {
      ph = sc.phase;
      sc.total[ph] = b;
    }
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    cl.sync();  // every block's total is written, with every write made before the call
    if (threadIdx.x == 0) {
      double s = 0;
      for (int r = 0; r < CL; r++) s += cl.map_shared_rank(sc.total, r)[ph];
      *reinterpret_cast<S*>(sc.out) = f(s);
      sc.phase = ph ^ 1;
    }
    // A block barrier publishes out.  The slot just read is written again two
    // sums later, after the next sum's cluster barrier, which no block passes
    // before every block has finished reading it.
    __syncthreads();
    return *reinterpret_cast<const S*>(sc.out);
  }
  static constexpr bool kCluster = true;
  // every block of the cluster starts with the same slot
  __device__ static void init() {
    if (threadIdx.x == 0) team_scratch().phase = 0;
  }
  __device__ static double sum(double v) { return sum_then(v, [](double t) { return t; }); }
  __device__ static int broadcast(const int* next) {
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    cl.sync();
    const int q = *cl.map_shared_rank(next, 0);
    cl.sync();
    return q;
  }
};

// ---------------------------------------------------------------------------
// Two blocks of a 4-block cluster, cluster ranks 2k and 2k + 1, running one
// chain while the other two run another (a cluster instance's middle class of
// chains, between the 4-block and the one-block ones).  The cluster barrier
// would tie the two pairs together, so each block has an mbarrier of two
// arrivals per phase: its own, and its partner's, made remotely through
// distributed shared memory.  A block's phase k + 1 cannot complete before
// its own arrival k + 1, which follows its wait for phase k, so the partner
// can never run two phases ahead.  Arrivals release and the wait acquires at
// cluster scope, ordering the blocks' global and shared memory accesses.  The
// wait is bounded; a block that gives up counts it, the chain's result is
// marked TG_E_TIMEOUT, and the GPU stays usable.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long* pair_mbar() {
  __shared__ __align__(8) unsigned long long m;
  return &m;
}
__device__ __forceinline__ unsigned& pair_parity() {
  __shared__ unsigned p;
  return p;
}
__device__ __forceinline__ int& pair_timeouts() {
  __shared__ int t;
  return t;
}
// at kernel start, thread 0 of every block; a cluster barrier must follow
// before any block arrives remotely
__device__ __forceinline__ void pair_barrier_init() {
  const unsigned a = (unsigned)__cvta_generic_to_shared(pair_mbar());
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 2;" ::"r"(a) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  pair_parity() = 0;
  pair_timeouts() = 0;
}
__device__ __forceinline__ void pair_barrier() {
  __syncthreads();  // the block's writes before thread 0's arrival
  if (threadIdx.x == 0) {
    const unsigned own = (unsigned)__cvta_generic_to_shared(pair_mbar());
    const unsigned partner = cooperative_groups::this_cluster().block_rank() ^ 1u;
    unsigned remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(own), "r"(partner));
    unsigned long long state;
    asm volatile("mbarrier.arrive.release.cluster.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(own) : "memory");
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(remote) : "memory");
    const unsigned parity = pair_parity();
    unsigned done = 0;
    for (int i = 0; i < (1 << 20) && !done; i++) {  // each try may suspend the thread briefly
      asm volatile(
          "{\n\t.reg .pred p;\n\t"
          "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(done)
          : "r"(own), "r"(parity)
          : "memory");
    }
    if (!done) pair_timeouts() += 1;
    pair_parity() = parity ^ 1u;
    (void)state;
  }
  __syncthreads();
}

struct PairTeam {
  __device__ static int rank() { return (int)(cooperative_groups::this_cluster().block_rank() & 1u); }
  __device__ static int nblocks() { return 2; }
  __device__ static void sync() { pair_barrier(); }
  template <typename P, class F> __device__ static auto sum_then(P v, F f) -> decltype(f(0.0)) {
    using S = decltype(f(0.0));
    static_assert(sizeof(S) <= sizeof(TeamScratch::out), "sum_then result too large");
    TeamScratch& sc = team_scratch();
    const double b = block_total_warp0(v, sc);
    int ph = 0;
    if (threadIdx.x == 0) {
      ph = sc.phase;
      sc.total[ph] = b;
    }
    pair_barrier();  // both totals written
    if (threadIdx.x == 0) {
      cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
      const double mine = sc.total[ph];
      const double other = cl.map_shared_rank(sc.total, cl.block_rank() ^ 1u)[ph];
      const double s = (rank() == 0) ? mine + other : other + mine;  // pair rank 0's total first
      *reinterpret_cast<S*>(sc.out) = f(s);
      sc.phase = ph ^ 1;
    }
    // as in ClusterTeam: the slot just read is written again two sums later,
    // after the next sum's pair barrier
    __syncthreads();
    return *reinterpret_cast<const S*>(sc.out);
  }
  static constexpr bool kCluster = false;
  __device__ static void init() {}
  __device__ static double sum(double v) { return sum_then(v, [](double t) { return t; }); }
  // the ticket pair rank 0's thread 0 wrote to `next`
  __device__ static int broadcast(const int* next) {
    pair_barrier();
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    const int q = (rank() == 0) ? *next : *cl.map_shared_rank(next, cl.block_rank() ^ 1u);
    pair_barrier();
    return q;
  }
};

// the chain's sites, split over the whole team
#define TG_BSITES(s, n) \
  for (int s = T::rank() * (int)blockDim.x + (int)threadIdx.x; s < (n); s += T::nblocks() * (int)blockDim.x)

struct ChainCtx {
  Geo g;
  double m, gc, mu, ep, em;
  int bc_t, bc_x;
  unsigned long long seed;
  // this chain's slices of the packed fields
  double2 *A, *An, *mom, *phi, *noise, *x, *Mx, *tmp, *Wt, *Wx, *r64, *p64, *p64b, *Mp64;
  float2 *Wt32, *Wx32, *xs, *rs, *ps, *ps2, *Mps;
};

struct CgOut {
  int iter, status, n_ru;
};

// What the CG loops need after the |r|^2 sum: the sum, beta, and the verdict
// of the stopping tests (FP64: a status, or -1 to go on; mixed: whether a
// reliable update is due, which runs the tests on the true residual).
struct CgTail64 {
  double rn, beta;
  int status;
};
struct CgTailMx {
  double rn;
  float fb;
  int need;
};

// ---------------------------------------------------------------------------
// CG on M^dag M inside one block.  Same recurrences, stopping rules and
// reliable-update rules as the single-lattice solver (tg_kernels.cu): p is
// formed as p = r + beta p at the top of each iteration (beta = 0 first and
// after a restart), pAp = |Mp|^2.
// ---------------------------------------------------------------------------
template <bool MU0, class T>
__device__ CgOut block_cg64(const ChainCtx& c, const BatchCg& P, const double2* b, double2* x) {
  const int V = c.g.V;
  OpK<double> km{c.m, c.ep, -c.em, MU0}, kd{c.m, -c.em, c.ep, MU0};
  double a = 0;
  TG_BSITES(s, V) {
    double2 bb = b[s];
    x[s] = make_double2(0, 0);
    c.r64[s] = bb;
    c.p64[s] = bb;
    a += bb.x * bb.x + bb.y * bb.y;
  }
  const double rr0 = T::sum(a);
  double stop = P.abs_tol2;
  if (P.rel_tol > 0 && P.rel_tol * P.rel_tol * rr0 > stop) stop = P.rel_tol * P.rel_tol * rr0;
  CgOut out{0, TG_OK, 0};
  if (!(rr0 >= stop) || rr0 == 0.0) {
    out.status = isnan(rr0) ? TG_E_NAN : TG_OK;
    return out;
  }
  double rr = rr0, beta = 0;
  int half = 0;
  while (true) {
    // p' = r + beta p formed where the stencil reads it (p of the previous
    // iteration in one buffer, p' stored at its own site in the other)
    const double2* p_old = half ? c.p64b : c.p64;
    double2* p_new = half ? c.p64 : c.p64b;
    double v = 0;
    auto ld = [&](int i) {
      const double2 rv = c.r64[i], pv = p_old[i];
      return make_double2(fma(beta, pv.x, rv.x), fma(beta, pv.y, rv.y));
    };
    auto epi = [&](int s, double2 o, double2 pc) {
      p_new[s] = pc;
      c.Mp64[s] = o;
      v = fma(o.x, o.x, v);
      v = fma(o.y, o.y, v);
    };
    stencil_team<T, double, 0, MU0>(c.g, km, ld, c.Wt, c.Wx, epi);
    const double alpha = T::sum_then(v, [&](double pAp) { return rr / pAp; });
    v = 0;
    auto ld2 = [&](int i) { return c.Mp64[i]; };
    auto epi2 = [&](int s, double2 ap, double2) {
      double2 xv = x[s], pv = p_new[s], rv = c.r64[s];
      xv.x += alpha * pv.x;
      xv.y += alpha * pv.y;
      rv.x -= alpha * ap.x;
      rv.y -= alpha * ap.y;
      x[s] = xv;
      c.r64[s] = rv;
      v = fma(rv.x, rv.x, v);
      v = fma(rv.y, rv.y, v);
    };
    stencil_team<T, double, 1, MU0>(c.g, kd, ld2, c.Wt, c.Wx, epi2);
    const CgTail64 e = T::sum_then(v, [&](double rn) {
      CgTail64 o{rn, rn / rr, -1};
      if (isnan(rn)) o.status = TG_E_NAN;
      else if (rn < stop) o.status = TG_OK;
      else if (rn / rr0 > 1e10) o.status = TG_E_DIVERGED;
      else if (out.iter + 1 >= P.maxiter) o.status = TG_E_NOCONV;
      return o;
    });
    half ^= 1;
    out.iter++;
    beta = e.beta;
    rr = e.rn;
    if (e.status >= 0) {
      out.status = e.status;
      break;
    }
  }
  T::sync();
  return out;
}

template <bool MU0, class T>
__device__ CgOut block_cg_mixed(const ChainCtx& c, const BatchCg& P, const double2* b, double2* x) {
  const int V = c.g.V;
  OpK<double> km{c.m, c.ep, -c.em, MU0}, kd{c.m, -c.em, c.ep, MU0};
  OpK<float> km32{(float)c.m, (float)c.ep, (float)-c.em, MU0}, kd32{(float)c.m, (float)-c.em, (float)c.ep, MU0};
  double a = 0;
  TG_BSITES(s, V) {
    double2 bb = b[s];
    x[s] = make_double2(0, 0);
    float2 rb = make_float2((float)bb.x, (float)bb.y);
    c.rs[s] = rb;
    c.ps[s] = rb;
    c.xs[s] = make_float2(0.f, 0.f);
    a += bb.x * bb.x + bb.y * bb.y;
  }
  const double rr0 = T::sum(a);
  double stop = P.abs_tol2;
  if (P.rel_tol > 0 && P.rel_tol * P.rel_tol * rr0 > stop) stop = P.rel_tol * P.rel_tol * rr0;
  CgOut out{0, TG_OK, 0};
  if (!(rr0 >= stop) || rr0 == 0.0) {
    out.status = isnan(rr0) ? TG_E_NAN : TG_OK;
    return out;
  }
  double rr = rr0, rr_true = rr0;
  float fb = 0.f;
  int since = 0, half = 0;
  // The FP32 iteration's operands, out of the shared-memory context: read
  // through it, every pointer would be reloaded for each row, since the
  // compiler cannot tell the rows' global stores from shared memory.
  const Geo g = c.g;
  float2* const rs = c.rs;
  float2* const xs = c.xs;
  float2* const Mps = c.Mps;
  float2* const ps_a = c.ps;
  float2* const ps_b = c.ps2;
  const float2* const Wt32 = c.Wt32;
  const float2* const Wx32 = c.Wx32;
  while (true) {
    const float2* p_old = half ? ps_b : ps_a;
    float2* p_new = half ? ps_a : ps_b;
    float v = 0;
    auto ld = [&](int i) {
      const float2 rv = rs[i], pv = p_old[i];
      return make_float2(fmaf(fb, pv.x, rv.x), fmaf(fb, pv.y, rv.y));
    };
    auto epi = [&](int s, float2 o, float2 pc) {
      p_new[s] = pc;
      Mps[s] = o;
      v = fmaf(o.x, o.x, v);
      v = fmaf(o.y, o.y, v);
    };
    stencil_team<T, float, 0, MU0>(g, km32, ld, Wt32, Wx32, epi);
    const float fa = T::sum_then(v, [&](double pAp) { return (float)(rr / pAp); });
    v = 0;
    auto ld2 = [&](int i) { return Mps[i]; };
    auto epi2 = [&](int s, float2 ap, float2) {
      float2 xv = xs[s], pv = p_new[s], rv = rs[s];
      xv.x = fmaf(fa, pv.x, xv.x);
      xv.y = fmaf(fa, pv.y, xv.y);
      rv.x = fmaf(-fa, ap.x, rv.x);
      rv.y = fmaf(-fa, ap.y, rv.y);
      xs[s] = xv;
      rs[s] = rv;
      v = fmaf(rv.x, rv.x, v);
      v = fmaf(rv.y, rv.y, v);
    };
    stencil_team<T, float, 1, MU0>(g, kd32, ld2, Wt32, Wx32, epi2);
    const CgTailMx e = T::sum_then(v, [&](double rn) {
      CgTailMx o{rn, (float)(rn / rr), 0};
      o.need = since + 1 >= P.ru_interval || rn < stop || rn < kRuDrop * rr_true || out.iter + 1 >= P.maxiter ||
               rn / rr0 > 1e10 || isnan(rn);
      return o;
    });
    half ^= 1;
    out.iter++;
    since++;
    fb = e.fb;
    rr = e.rn;
    if (!e.need) continue;
    // reliable update: x += xs, r = b - M^dag M x in FP64
    TG_BSITES(s, V) {
      float2 d = c.xs[s];
      double2 xv = x[s];
      xv.x += (double)d.x;
      xv.y += (double)d.y;
      x[s] = xv;
      c.xs[s] = make_float2(0.f, 0.f);
    }
    T::sync();
    TG_BSITES(s, V) c.tmp[s] = dslash_at<double, 0, MU0>(c.g, km, x, c.Wt, c.Wx, s);
    T::sync();
    double a2 = 0;
    TG_BSITES(s, V) {
      double2 ap = dslash_at<double, 1, MU0>(c.g, kd, c.tmp, c.Wt, c.Wx, s);
      double2 bb = b[s];
      double2 rv = make_double2(bb.x - ap.x, bb.y - ap.y);
      c.rs[s] = make_float2((float)rv.x, (float)rv.y);
      a2 = fma(rv.x, rv.x, a2);
      a2 = fma(rv.y, rv.y, a2);
    }
    const double rt = T::sum(a2);
    if (rt > kRuRestart * rr) fb = 0.f;  // recursive residual far too optimistic: restart p from r
    rr = rt;
    rr_true = rt;
    since = 0;
    out.n_ru++;
    if (isnan(rt)) { out.status = TG_E_NAN; break; }
    if (rt < stop) { out.status = TG_OK; break; }
    if (rt / rr0 > 1e10) { out.status = TG_E_DIVERGED; break; }
    if (out.iter >= P.maxiter) { out.status = TG_E_NOCONV; break; }
  }
  T::sync();
  return out;
}

template <bool MU0, class T>
__device__ __forceinline__ CgOut block_cg(const ChainCtx& c, const BatchCg& P, const double2* b, double2* x) {
  return P.precision == TG_PREC_MIXED ? block_cg_mixed<MU0, T>(c, P, b, x) : block_cg64<MU0, T>(c, P, b, x);
}

// ---------------------------------------------------------------------------
// One trajectory of one chain (update_gauge, hmc.c:671-746), by one block.
// ---------------------------------------------------------------------------
template <bool MU0, class T>
__device__ void chain_trajectory(const ChainCtx& c, const BatchTraj& P, ChainResult* res) {
  const int V = c.g.V;
  const Geo& g = c.g;
  OpK<double> km{c.m, c.ep, -c.em, MU0}, kd{c.m, -c.em, c.ep, MU0};
  const unsigned long long tr = res->traj;
  const bool noise_on = P.stochastic_term != 0;
  const double fac = kNf / c.gc;
  // refresh: links of A, eta (stream 0), momenta (16), noise (17); hmc.c:695-699
  double a_pf = 0, a_mom = 0, a_g = 0;
  TG_BSITES(s, V) {
    double2 a = c.A[s];
    write_links(g, c.bc_t, c.bc_x, s, a, c.Wt, c.Wx, c.Wt32, c.Wx32);
    double2 e = philox_gauss_pair(c.seed, tr, (unsigned)s, 0u);
    c.tmp[s] = e;
    a_pf += e.x * e.x + e.y * e.y;
    double2 p = philox_gauss_pair(c.seed, tr, (unsigned)s, 16u);
    c.mom[s] = p;
    a_mom += p.x * p.x + p.y * p.y;
    a_g += (1. - cos(a.x)) + (1. - cos(a.y));
    if (noise_on) c.noise[s] = philox_gauss_pair(c.seed, tr, (unsigned)s, 17u);
    c.An[s] = a;
  }
  const double Spf0 = T::sum(a_pf), Smom0 = T::sum(a_mom), Sg0 = fac * T::sum(a_g);
  double a_md = 0;
  TG_BSITES(s, V) {
    c.phi[s] = dslash_at<double, 1, MU0>(g, kd, c.tmp, c.Wt, c.Wx, s);  // phi = M^dag eta
    if (noise_on) {
      double2 o = dslash_at<double, 1, MU0>(g, kd, c.noise, c.Wt, c.Wx, s);
      double2 n = c.noise[s];
      a_md += n.x * o.x + n.y * o.y;
    }
  }
  const double Smd0 = T::sum(a_md);
  // leapfrog, hmc.c:708-716 (two half steps between MD steps share a pass)
  const double eps = P.tau / P.nsteps;
  const double cstep = 2.0 * (P.tau * 0.5 / P.nsteps);
  const double gfac = eps * kNf / c.gc;
  int iters = 0, maxit = 0, n_ru = 0, status = TG_OK;
  for (int i = 0; i <= P.nsteps; i++) {
    const int nadd = (i == 0 || i == P.nsteps) ? 1 : 2;
    TG_BSITES(s, V) {
      double2 a = c.An[s], p = c.mom[s];
      for (int k = 0; k < nadd; k++) {
        a.x = __dadd_rn(a.x, __dmul_rn(cstep, p.x));
        a.y = __dadd_rn(a.y, __dmul_rn(cstep, p.y));
      }
      c.An[s] = a;
      write_links(g, c.bc_t, c.bc_x, s, a, c.Wt, c.Wx, c.Wt32, c.Wx32);
    }
    T::sync();
    CgOut o = block_cg<MU0, T>(c, P.cg, c.phi, c.x);
    iters += o.iter;
    maxit = max(maxit, o.iter);
    n_ru += o.n_ru;
    status = max(status, o.status);
    if (i == P.nsteps) break;  // the last solve gives S_pf at the end
    // M x: a mixed solve ends on a reliable update, which left M x of the final x
    // in tmp (the same function of the same operands); otherwise apply M.
    const double2* Mx = c.tmp;
    if (P.cg.precision != TG_PREC_MIXED || o.n_ru == 0) {
      TG_BSITES(s, V) c.Mx[s] = dslash_at<double, 0, MU0>(g, km, c.x, c.Wt, c.Wx, s);
      T::sync();
      Mx = c.Mx;
    }
    TG_BSITES(s, V) {
      ForcePieces f = force_site(g, c.bc_t, c.bc_x, c.ep, c.em, c.An, c.Wt, c.Wx, c.x, Mx,
                                 noise_on ? c.noise : nullptr, s);
      double2 p = c.mom[s];
      p.x -= gfac * f.g.x;
      p.y -= gfac * f.g.y;
      p.x -= eps * f.pf.x;
      p.y -= eps * f.pf.y;
      if (noise_on) {
        p.x -= eps * f.md.x;
        p.y -= eps * f.md.y;
      }
      c.mom[s] = p;
    }
    T::sync();
  }
  // end actions, hmc.c:719-726
  double b_pf = 0, b_mom = 0, b_g = 0, b_md = 0;
  TG_BSITES(s, V) {
    double2 ph = c.phi[s], xv = c.x[s], p = c.mom[s], a = c.An[s];
    b_pf += ph.x * xv.x + ph.y * xv.y;
    b_mom += p.x * p.x + p.y * p.y;
    b_g += (1. - cos(a.x)) + (1. - cos(a.y));
    if (noise_on) {
      double2 o = dslash_at<double, 1, MU0>(g, kd, c.noise, c.Wt, c.Wx, s);
      double2 n = c.noise[s];
      b_md += n.x * o.x + n.y * o.y;
    }
  }
  const double Spf1 = T::sum(b_pf), Smom1 = T::sum(b_mom), Sg1 = fac * T::sum(b_g), Smd1 = T::sum(b_md);
  const double dS = Smom1 - Smom0 + Spf1 - Spf0 + Smd1 - Smd0 + Sg1 - Sg0;  // hmc.c:729-732
  const double u = philox_uniform1(c.seed, tr, 18u);
  const int acc = exp(-dS) > u ? 1 : 0;  // hmc.c:738
  if (acc) TG_BSITES(s, V) c.A[s] = c.An[s];
  if (T::rank() == 0 && threadIdx.x == 0) {
    res->dH = dS;
    res->Sg0 = Sg0; res->Spf0 = Spf0; res->Smd0 = Smd0; res->Smom0 = Smom0;
    res->Sg1 = Sg1; res->Spf1 = Spf1; res->Smd1 = Smd1; res->Smom1 = Smom1;
    res->u = u;
    res->accepted = acc;
    res->status = status;
    res->cg_iterations = iters;
    res->cg_max_iterations = maxit;
    res->reliable_updates = n_ru;
    res->solves = P.nsteps + 1;
    res->traj = tr + 1;
  }
  T::sync();
}

__device__ __forceinline__ void fill_ctx(ChainCtx& c, const BatchChain& b, const BatchFields& F) {
    c.g = b.geo;
    c.m = b.m;
    c.gc = b.g;
    c.mu = b.mu;
    c.ep = exp(b.mu);
    c.em = exp(-b.mu);
    c.bc_t = b.bc_t;
    c.bc_x = b.bc_x;
    c.seed = b.seed;
    const long long o = b.off;
    c.A = F.A + o; c.An = F.An + o; c.mom = F.mom + o; c.phi = F.phi + o; c.noise = F.noise + o;
    c.x = F.x + o; c.Mx = F.Mx + o; c.tmp = F.tmp + o; c.Wt = F.Wt + o; c.Wx = F.Wx + o;
    c.r64 = F.r64 + o; c.p64 = F.p64 + o; c.p64b = F.p64b + o; c.Mp64 = F.Mp64 + o;
    c.Wt32 = F.Wt32 + o; c.Wx32 = F.Wx32 + o; c.xs = F.xs + o; c.rs = F.rs + o; c.ps = F.ps + o;
    c.ps2 = F.ps2 + o; c.Mps = F.Mps + o;
}

// The two ends of the work queue (one 64-bit word: front draws in the low
// half, back draws in the high half).  A draw succeeds while front + back < n
// before it: in the word's order of updates every position is then handed out
// once, to whichever end reaches it first.  Both return n when nothing is left.
__device__ __forceinline__ int queue_front(unsigned long long* queue, int n) {
  const unsigned long long old = atomicAdd(queue, 1ull);
  const long long f = (long long)(old & 0xffffffffull), b = (long long)(old >> 32);
  return (f + b < n) ? (int)f : n;
}
// From the back, but only positions at or after `lo`: the test and the draw are
// one compare-and-swap, so a refused position stays with the front.  The
// retries are bounded; a block that gives up leaves the rest to the front.
__device__ __forceinline__ int queue_back(unsigned long long* queue, int n, int lo) {
  unsigned long long old = *reinterpret_cast<volatile unsigned long long*>(queue);
  for (int tries = 0; tries < (1 << 20); tries++) {
    const long long f = (long long)(old & 0xffffffffull), b = (long long)(old >> 32);
    const long long t = (long long)n - 1 - b;
    if (f + b >= n || t < lo) return n;
    const unsigned long long seen = atomicCAS(queue, old, old + (1ull << 32));
    if (seen == old) return (int)t;
    old = seen;
  }
  return n;
}

template <int BS, int MINB, class T, bool PAIRS = false>
__device__ __forceinline__ void batch_trajectory_body(const BatchChain* __restrict__ chains,
                                                      const int* __restrict__ order, int n, const BatchFields& F,
                                                      const BatchTraj& P, ChainResult* results,
                                                      unsigned long long* queue) {
  // The chain context (geometry, couplings, ~20 field pointers) lives in shared
  // memory: kept in registers it would cost ~40 of them per thread.  Every
  // block of a team fills its own copy.
  __shared__ int next;
  __shared__ ChainCtx c;
  if constexpr (PAIRS) {
    if (threadIdx.x == 0) pair_barrier_init();
  }
  T::init();  // published by the first broadcast's barriers
  int q;
  while (true) {
    if (T::rank() == 0 && threadIdx.x == 0)
      next = (!T::kCluster && P.from_back) ? queue_back(queue, n, P.solo_from) : queue_front(queue, n);
    q = T::broadcast(&next);
    if (q >= n || (T::kCluster && q >= P.solo_from)) break;
    const int ci = order[q];
    if (threadIdx.x == 0) fill_ctx(c, chains[ci], F);
    __syncthreads();
    if (c.mu == 0.0) chain_trajectory<true, T>(c, P, &results[ci]);
    else chain_trajectory<false, T>(c, P, &results[ci]);
  }
  if constexpr (T::kCluster) {
    int carry = -1;  // a ticket past pair_end that this block runs alone
    if constexpr (PAIRS) {
      // Queue positions [solo_from, pair_end): the cluster splits into two
      // pairs; ranks 0-1 run chain q, ranks 2-3 take the next.  A pair whose
      // ticket lies past pair_end splits again: its rank 0 runs that chain
      // alone.  (The broadcast's closing cluster barrier has ordered every
      // earlier access; each pair's blocks touch only each other's shared
      // memory.)
      if (q < n && q < P.pair_end) {
        const bool first = (cooperative_groups::this_cluster().block_rank() >> 1) == 0;
        int pq = first ? q : -1;
        while (true) {
          if (pq < 0) {
            if (PairTeam::rank() == 0 && threadIdx.x == 0) next = queue_front(queue, n);
            pq = PairTeam::broadcast(&next);
          }
          if (pq >= n) break;
          if (pq >= P.pair_end) {
            if (PairTeam::rank() == 0) carry = pq;
            break;
          }
          const int ci = order[pq];
          if (threadIdx.x == 0) {
            fill_ctx(c, chains[ci], F);
            pair_timeouts() = 0;
          }
          __syncthreads();
          if (c.mu == 0.0) chain_trajectory<true, PairTeam>(c, P, &results[ci]);
          else chain_trajectory<false, PairTeam>(c, P, &results[ci]);
          if (PairTeam::rank() == 0 && threadIdx.x == 0 && pair_timeouts() > 0) results[ci].status = TG_E_TIMEOUT;
          pq = -1;
        }
        q = n;  // q was run by a pair
      }
    }
    // The rest of the queue holds small chains: rank 0 runs chain q and every
    // block then takes chains of its own, with block barriers only.  No block
    // touches another's shared memory from here on (the broadcast's closing
    // cluster barrier has ordered every earlier access).
    int mine = (q < n && T::rank() == 0) ? q : carry;
    while (true) {
      if (mine < 0) {
        if (threadIdx.x == 0) next = queue_front(queue, n);
        __syncthreads();
        mine = next;
        if (mine >= n) break;
      }
      const int ci = order[mine];
      if (threadIdx.x == 0) fill_ctx(c, chains[ci], F);
      __syncthreads();
      if (c.mu == 0.0) chain_trajectory<true, BlockTeam>(c, P, &results[ci]);
      else chain_trajectory<false, BlockTeam>(c, P, &results[ci]);
      mine = -1;
    }
  }
}

}  // namespace tg
