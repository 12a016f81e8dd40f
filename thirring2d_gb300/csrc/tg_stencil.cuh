// tg_stencil.cuh -- the warp column march of the staggered operator, shared
// by the launch-per-iteration kernels (tg_kernels.cu) and the persistent
// solver (tg_pcg.cu), in two forms:
//   march_segment         operands loaded into registers as the march needs them
//   march_segment_staged  rows of the next chunks staged in shared memory by
//                         TMA bulk copies (cp.async.bulk + mbarrier) while the
//                         current chunk computes
#pragma once

#include "tg_device.cuh"

namespace tg {

// One row t of a warp's march: the operator at the 32 sites (t, x0 + lane)
// from psi(t-1) = pm, psi(t) = pc, psi(t+1) = pp and the links, with the
// operand across the warp's edge pe (used by lanes 0 and 31) and the x link
// entering column x0 we (used by lane 0).  Rotates pm, pc, wtm for row t+1.
template <typename R, int DAG, bool MU0, bool UNIT, class Epi>
__device__ __forceinline__ void march_row(const OpK<R>& k, int s, int lane, C2<R>& pm, C2<R>& pc, C2<R>& wtm,
                                          C2<R> pp, C2<R> wt, C2<R> wx, C2<R> pe, C2<R> we, Epi& epi) {
  C2<R> pr = shfl_down1<R>(pc);
  C2<R> pl = shfl_up1<R>(pc);
  C2<R> wl = shfl_up1<R>(wx);
  if (lane == 31) pr = pe;
  if (lane == 0) {
    pl = pe;
    wl = we;
  }
  epi(s, dslash_vals<R, DAG, MU0, UNIT>(k, pc, pp, pm, pr, pl, wt, wtm, wx, wl), pc);
  pm = pc;
  pc = pp;
  wtm = wt;
}

template <typename R> __device__ __forceinline__ C2<R> shfl_c2(C2<R> v, int src) {
  return mk<R>(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// The operands across the warp's two edges for rows t .. t+kMarchT-1, fetched
// once by the first lanes: lane i < kMarchT the operand left of x0 in row t+i
// (and, in ew, the x link entering x0), lane kMarchT+i the operand right of
// x0+31.  Shuffles later hand them to lanes 0 and 31, so no lane fetches (or
// recombines) an operand it does not use.
template <typename R, class Ld>
__device__ __forceinline__ void edge_operands(const Geo& g, Ld& ld, const C2<R>* __restrict__ Wx, int t, int xle,
                                              int xre, int lane, C2<R>& ep, C2<R>& ew) {
  ep = mk<R>(0, 0);
  ew = mk<R>(0, 0);
  if (lane < 2 * kMarchT) {
    const int rr = t + (lane < kMarchT ? lane : lane - kMarchT);
    ep = ld(rr * g.nx + (lane < kMarchT ? xle : xre));
    if (lane < kMarchT) ew = Wx[rr * g.nx + xle];
  }
}

// One warp marches rows ta .. tb-1 (tb > ta) of the 32 columns x0 = 32*xw ..
// x0+31, lane = column.  ld(i) yields the operand at site i (a plain load, or a
// vector recombined on the fly); epi(s, out(s), operand(s)) consumes each
// site's result.  psi(t-1), psi(t) and Wt(t-1) stay in registers from row to
// row; x neighbours come from warp shuffles.
template <typename R, int DAG, bool MU0, bool UNIT = false, class Ld, class Epi>
__device__ __forceinline__ void march_segment(const Geo& g, const OpK<R>& k, Ld& ld, const C2<R>* __restrict__ Wt,
                                              const C2<R>* __restrict__ Wx, int xw, int ta, int tb, Epi& epi) {
  const int nx = g.nx;
  const int lane = threadIdx.x & 31;
  const int x0 = xw << 5;
  const int x = x0 + lane;
  const int xle = (x0 == 0) ? nx - 1 : x0 - 1;       // column left of the warp
  const int xre = (x0 + 32 == nx) ? 0 : x0 + 32;     // column right of the warp
  const int tm = (ta == 0) ? g.nt - 1 : ta - 1;
  C2<R> pm = ld(tm * nx + x);
  C2<R> wtm = Wt[tm * nx + x];
  C2<R> pc = ld(ta * nx + x);
  auto row = [&](int t, C2<R> pe, C2<R> we) {
    const int tp = (t + 1 == g.nt) ? 0 : t + 1;
    const int s = t * nx + x;
    march_row<R, DAG, MU0, UNIT>(k, s, lane, pm, pc, wtm, ld(tp * nx + x), Wt[s], Wx[s], pe, we, epi);
  };
  int t = ta;
  for (; t + kMarchT <= tb; t += kMarchT) {
    C2<R> ep, ew;
    edge_operands<R>(g, ld, Wx, t, xle, xre, lane, ep, ew);
    if constexpr (sizeof(R) == 4) {
      // FP32 (memory- or latency-bound): every load of the chunk is issued
      // before its first result is stored.  The epilogue's stores may alias the
      // operands as far as the compiler knows, and would otherwise hold each
      // row's loads behind the previous row's stores, one memory latency per
      // row.  (The FP64 march is bound by the FP64 pipe and keeps its
      // registers.)
      C2<R> pp[kMarchT], wt[kMarchT], wx[kMarchT];
#pragma unroll
      for (int i = 0; i < kMarchT; i++) {
        const int tt = t + i;
        const int tp = (tt + 1 == g.nt) ? 0 : tt + 1;
        pp[i] = ld(tp * nx + x);
        wt[i] = Wt[tt * nx + x];
        wx[i] = Wx[tt * nx + x];
      }
#pragma unroll
      for (int i = 0; i < kMarchT; i++)
        march_row<R, DAG, MU0, UNIT>(k, (t + i) * nx + x, lane, pm, pc, wtm, pp[i], wt[i], wx[i],
                                     shfl_c2<R>(ep, (lane == 31) ? kMarchT + i : i), shfl_c2<R>(ew, i), epi);
    } else {
#pragma unroll
      for (int i = 0; i < kMarchT; i++) row(t + i, shfl_c2<R>(ep, (lane == 31) ? kMarchT + i : i), shfl_c2<R>(ew, i));
    }
  }
  for (; t < tb; t++) {  // the last rows of the segment: lanes 0 and 31 fetch their own
    const int xe = (lane == 31) ? xre : xle;
    row(t, ld(t * nx + xe), Wx[t * nx + xle]);
  }
}

// The (strip, t) rows of the lattice in strip-major order, split into one
// contiguous range per warp: ranges differ by at most one row, and a warp
// restarts its march only where its range crosses into a new strip.  Calls
// f(xw, ta, tb) for each strip segment of this warp's range.
template <class F> __device__ __forceinline__ void for_warp_rows(const Geo& g, F&& f) {
  const int wpb = (int)(blockDim.x >> 5);
  const long long rows = (long long)(g.nx >> 5) * g.nt;
  const long long nw = (long long)gridDim.x * wpb;
  const long long gw = (long long)blockIdx.x * wpb + (threadIdx.x >> 5);
  long long r = rows * gw / nw;
  const long long r1 = rows * (gw + 1) / nw;
  while (r < r1) {
    const int xw = (int)(r / g.nt);
    const int ta = (int)(r - (long long)xw * g.nt);
    const int tb = (r1 - r < (long long)(g.nt - ta)) ? ta + (int)(r1 - r) : g.nt;
    f(xw, ta, tb);
    r += tb - ta;
  }
}

// Apply the operator to every site and hand each result to epi: column march
// where the lattice allows it, else one site per thread.
template <typename R, int DAG, bool MU0, bool UNIT = false, class Ld, class Epi>
__device__ __forceinline__ void stencil_ld(const Geo& g, const OpK<R>& k, Ld& ld, const C2<R>* __restrict__ Wt,
                                           const C2<R>* __restrict__ Wx, Epi& epi) {
  if (g.march) {
    for_warp_rows(g, [&](int xw, int ta, int tb) { march_segment<R, DAG, MU0, UNIT>(g, k, ld, Wt, Wx, xw, ta, tb, epi); });
  } else {
    TG_SITES(s, g.V) {
      int t, x;
      site_tx(g, s, t, x);
      const Nbr n = neighbours(g, s, t, x);
      const C2<R> pc = ld(s);
      epi(s, dslash_vals<R, DAG, MU0, UNIT>(k, pc, ld(n.tp), ld(n.tm), ld(n.xp), ld(n.xm), Wt[s], Wt[n.tm], Wx[s],
                                            Wx[n.xm]),
          pc);
    }
  }
}

template <typename R, int DAG, bool MU0, bool UNIT = false, class Epi>
__device__ __forceinline__ void stencil_all(const Geo& g, const OpK<R>& k, const C2<R>* __restrict__ in,
                                            const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx, Epi& epi) {
  auto ld = [&](int i) { return in[i]; };
  stencil_ld<R, DAG, MU0, UNIT>(g, k, ld, Wt, Wx, epi);
}

// The operator over one small lattice run by a team of thread blocks (the
// batched-chain kernel: one block, or the blocks of a cluster).  T gives the
// block's rank in the team and the team's size.  The team's warps split the
// lattice's (strip, t) rows into one contiguous range each, as for_warp_rows
// splits them over a grid; lattices whose nx is not a multiple of 32 go one
// site per thread.
template <class T, typename R, int DAG, bool MU0, class Ld, class Epi>
__device__ __forceinline__ void stencil_team(const Geo& g, const OpK<R>& k, Ld& ld, const C2<R>* __restrict__ Wt,
                                             const C2<R>* __restrict__ Wx, Epi& epi) {
  const int wpb = blockDim.x >> 5;
  if ((g.nx & 31) == 0) {
    const int nw = T::nblocks() * wpb, w = T::rank() * wpb + (threadIdx.x >> 5);
    const int rows = (g.nx >> 5) * g.nt;
    int r = (int)((long long)rows * w / nw);
    const int r1 = (int)((long long)rows * (w + 1) / nw);
    while (r < r1) {
      const int xw = r / g.nt;
      const int ta = r - xw * g.nt;
      const int tb = (r1 - r < g.nt - ta) ? ta + (r1 - r) : g.nt;
      march_segment<R, DAG, MU0>(g, k, ld, Wt, Wx, xw, ta, tb, epi);
      r += tb - ta;
    }
  } else {
    for (int s = T::rank() * (int)blockDim.x + (int)threadIdx.x; s < g.V; s += T::nblocks() * (int)blockDim.x) {
      int t, x;
      site_tx(g, s, t, x);
      const Nbr n = neighbours(g, s, t, x);
      const C2<R> pc = ld(s);
      epi(s, dslash_vals<R, DAG, MU0>(k, pc, ld(n.tp), ld(n.tm), ld(n.xp), ld(n.xm), Wt[s], Wt[n.tm], Wx[s], Wx[n.xm]),
          pc);
    }
  }
}

// Blocks of work of a stencil kernel (march: at least kMarchT rows per warp).
inline int stencil_work(const Geo& g) {
  return g.march ? ((g.nx >> 5) * ((g.nt + kMarchT - 1) / kMarchT) + kBlock / 32 - 1) / (kBlock / 32) : nblocks(g.V);
}

// ---------------------------------------------------------------------------
// TMA-staged march.  Each warp owns kStages stage buffers in dynamic shared
// memory, each holding one chunk (kMarchT rows) of its 32 columns: the
// operand sources of rows t+1 .. t+kMarchT and Wt, Wx of rows t .. t+kMarchT-1.
// Lane 0 fills a stage with one 32-site row segment per array and row
// (cp.async.bulk, 16-byte aligned because x0 is a multiple of 32) and arms
// the stage's mbarrier with the byte count; the warp waits on the barrier's
// phase, computes the chunk from shared memory, and lane 0 refills the stage
// with the chunk kStages ahead.  The operand of a site is combine() of its
// NSRC source arrays (one: a plain vector; two: r + beta p of CG).
// ---------------------------------------------------------------------------
template <typename R> struct SrcOne {  // the operand is a[i]
  static constexpr int n = 1;
  const C2<R>* a;
  __device__ __forceinline__ const C2<R>* arr(int) const { return a; }
  __device__ __forceinline__ C2<R> combine(const C2<R>* v) const { return v[0]; }
  __device__ __forceinline__ C2<R> operator()(int i) const { return a[i]; }
};

template <typename R> struct SrcAxpy {  // the operand is r[i] + beta p[i] (the CG direction p')
  static constexpr int n = 2;
  const C2<R>* r;
  const C2<R>* p;
  R beta;
  __device__ __forceinline__ const C2<R>* arr(int j) const { return j ? p : r; }
  __device__ __forceinline__ C2<R> combine(const C2<R>* v) const {
    return mk<R>(fma(beta, v[1].x, v[0].x), fma(beta, v[1].y, v[0].y));
  }
  __device__ __forceinline__ C2<R> operator()(int i) const {
    const C2<R> rv = r[i], pv = p[i];
    return mk<R>(fma(beta, pv.x, rv.x), fma(beta, pv.y, rv.y));
  }
};

template <int NSRC> struct StageShape {
  static constexpr int stages = NSRC == 1 ? 4 : 3;  // 12 rows ahead at most, 12 KB per warp in FP32
};
template <typename R, int NSRC> __host__ __device__ constexpr int stage_bytes() {
  return (NSRC + 2) * kMarchT * 32 * (int)sizeof(C2<R>);
}
// Dynamic shared memory of a staged kernel: every warp's stages, then their mbarriers.
template <typename R, int NSRC> __host__ __device__ constexpr int staged_smem_bytes() {
  return (kBlock / 32) * (StageShape<NSRC>::stages * stage_bytes<R, NSRC>() + StageShape<NSRC>::stages * 8);
}

// Waits on a stage's mbarrier are bounded: kStageWaitLimit polls of
// try_wait (each suspends for a hardware-chosen slice).  A wait that runs
// out counts in g_stage_faults and the chunk is computed from whatever the
// stage holds, so a fault shows as an error count and wrong numbers, never as
// a hung GPU.
constexpr int kStageWaitLimit = 1 << 22;
static __device__ unsigned g_stage_faults;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// generic-proxy accesses to shared memory before later TMA writes to it
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void stage_wait(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < kStageWaitLimit; it++)
    if (mbar_try_wait(bar, parity)) return;
  if ((threadIdx.x & 31) == 0) atomicAdd(&g_stage_faults, 1u);
}

template <typename R, int DAG, bool MU0, bool UNIT, class Src, class Epi>
__device__ __forceinline__ void march_segment_staged(const Geo& g, const OpK<R>& k, const Src& src,
                                                     const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx,
                                                     int xw, int ta, int tb, Epi& epi, unsigned char* stage,
                                                     unsigned long long* bars, unsigned& phases) {
  constexpr int NS = StageShape<Src::n>::stages;
  constexpr int RB = 32 * (int)sizeof(C2<R>);  // one row segment of one array
  constexpr int SB = stage_bytes<R, Src::n>();
  const int nx = g.nx;
  const int lane = threadIdx.x & 31;
  const int x0 = xw << 5;
  const int x = x0 + lane;
  const int xle = (x0 == 0) ? nx - 1 : x0 - 1;
  const int xre = (x0 + 32 == nx) ? 0 : x0 + 32;
  const int nchunks = (tb - ta) / kMarchT;
  // lane 0: chunk c (rows ta + c*kMarchT ..) into stage c % NS
  auto issue = [&](int c) {
    const int sg = c % NS;
    unsigned char* base = stage + sg * SB;
    const int t = ta + c * kMarchT;
    mbar_expect_tx(bars + sg, (unsigned)SB);
#pragma unroll
    for (int i = 0; i < kMarchT; i++) {
      const int tp = (t + i + 1 == g.nt) ? 0 : t + i + 1;
#pragma unroll
      for (int j = 0; j < Src::n; j++)
        bulk_g2s(base + (j * kMarchT + i) * RB, src.arr(j) + (size_t)tp * nx + x0, RB, bars + sg);
      bulk_g2s(base + (Src::n * kMarchT + i) * RB, Wt + (size_t)(t + i) * nx + x0, RB, bars + sg);
      bulk_g2s(base + ((Src::n + 1) * kMarchT + i) * RB, Wx + (size_t)(t + i) * nx + x0, RB, bars + sg);
    }
  };
  if (lane == 0) {
    fence_proxy_async_smem();
    for (int c = 0; c < nchunks && c < NS; c++) issue(c);
  }
  const int tm = (ta == 0) ? g.nt - 1 : ta - 1;
  C2<R> pm = src(tm * nx + x);
  C2<R> wtm = Wt[tm * nx + x];
  C2<R> pc = src(ta * nx + x);
  int t = ta;
  for (int c = 0; c < nchunks; c++, t += kMarchT) {
    const int sg = c % NS;
    C2<R> ep, ew;
    edge_operands<R>(g, src, Wx, t, xle, xre, lane, ep, ew);
    stage_wait(bars + sg, (phases >> sg) & 1u);
    phases ^= 1u << sg;
    const C2<R>* sv = reinterpret_cast<const C2<R>*>(stage + sg * SB);
#pragma unroll
    for (int i = 0; i < kMarchT; i++) {
      C2<R> v[Src::n];
#pragma unroll
      for (int j = 0; j < Src::n; j++) v[j] = sv[(j * kMarchT + i) * 32 + lane];
      march_row<R, DAG, MU0, UNIT>(k, (t + i) * nx + x, lane, pm, pc, wtm, src.combine(v),
                                   sv[(Src::n * kMarchT + i) * 32 + lane], sv[((Src::n + 1) * kMarchT + i) * 32 + lane],
                                   shfl_c2<R>(ep, (lane == 31) ? kMarchT + i : i), shfl_c2<R>(ew, i), epi);
    }
    __syncwarp();
    if (lane == 0 && c + NS < nchunks) {
      fence_proxy_async_smem();
      issue(c + NS);
    }
  }
  for (; t < tb; t++) {
    const int tp = (t + 1 == g.nt) ? 0 : t + 1;
    const int s = t * nx + x;
    const int xe = (lane == 31) ? xre : xle;
    march_row<R, DAG, MU0, UNIT>(k, s, lane, pm, pc, wtm, src(tp * nx + x), Wt[s], Wx[s], src(t * nx + xe),
                                 Wx[t * nx + xle], epi);
  }
}

// stencil_ld with the operand from Src, staged through shared memory on
// marching lattices.  The kernel must be launched with
// staged_smem_bytes<R, Src::n>() of dynamic shared memory.
template <typename R, int DAG, bool MU0, bool UNIT, class Src, class Epi>
__device__ __forceinline__ void stencil_staged(const Geo& g, const OpK<R>& k, const Src& src,
                                               const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx, Epi& epi) {
  if (!g.march) {
    Src ld = src;
    stencil_ld<R, DAG, MU0, UNIT>(g, k, ld, Wt, Wx, epi);
    return;
  }
  extern __shared__ __align__(128) unsigned char tg_dyn_smem[];
  constexpr int NS = StageShape<Src::n>::stages;
  constexpr int WB = NS * stage_bytes<R, Src::n>();
  const int w = threadIdx.x >> 5;
  unsigned char* stage = tg_dyn_smem + w * WB;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(tg_dyn_smem + (kBlock / 32) * WB) + w * NS;
  if ((threadIdx.x & 31) == 0) {
    for (int sg = 0; sg < NS; sg++) mbar_init(bars + sg, 1);
    mbar_init_fence();
  }
  __syncwarp();
  unsigned phases = 0;
  for_warp_rows(g, [&](int xw, int ta, int tb) {
    march_segment_staged<R, DAG, MU0, UNIT>(g, k, src, Wt, Wx, xw, ta, tb, epi, stage, bars, phases);
  });
}

}  // namespace tg
