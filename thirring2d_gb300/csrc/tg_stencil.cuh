// tg_stencil.cuh -- the warp column march of the staggered operator, shared
// by the launch-per-iteration kernels (tg_kernels.cu) and the persistent
// solver (tg_pcg.cu).
#pragma once

#include "tg_device.cuh"

namespace tg {

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
  // row t, given the operand across the warp's edge (pe: used by lanes 0 and
  // 31) and the x link entering column x0 (we: used by lane 0)
  auto row = [&](int t, C2<R> pe, C2<R> we) {
    const int tp = (t + 1 == g.nt) ? 0 : t + 1;
    const int s = t * nx + x;
    const C2<R> pp = ld(tp * nx + x);
    const C2<R> wt = Wt[s];
    const C2<R> wx = Wx[s];
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
  };
  int t = ta;
  for (; t + kMarchT <= tb; t += kMarchT) {
    // The edge operands of kMarchT rows, fetched once by the first lanes: lane
    // i < kMarchT the operand left of x0 in row t+i (and the x link entering
    // x0), lane kMarchT+i the operand right of x0+31.  Shuffles hand them to
    // lanes 0 and 31, so no lane fetches or recombines an operand it does not use.
    C2<R> ep = mk<R>(0, 0), ew = mk<R>(0, 0);
    if (lane < 2 * kMarchT) {
      const int rr = t + (lane < kMarchT ? lane : lane - kMarchT);
      ep = ld(rr * nx + (lane < kMarchT ? xle : xre));
      if (lane < kMarchT) ew = Wx[rr * nx + xle];
    }
#pragma unroll
    for (int i = 0; i < kMarchT; i++) {
      const int src = (lane == 31) ? kMarchT + i : i;
      row(t + i, mk<R>(__shfl_sync(0xffffffffu, ep.x, src), __shfl_sync(0xffffffffu, ep.y, src)),
          mk<R>(__shfl_sync(0xffffffffu, ew.x, i), __shfl_sync(0xffffffffu, ew.y, i)));
    }
  }
  for (; t < tb; t++) {  // the last rows of the segment: lanes 0 and 31 fetch their own
    const int xe = (lane == 31) ? xre : xle;
    row(t, ld(t * nx + xe), Wx[t * nx + xle]);
  }
}

// Apply the operator to every site and hand each result to epi: column march
// where the lattice allows it, else one site per thread.
template <typename R, int DAG, bool MU0, bool UNIT = false, class Ld, class Epi>
__device__ __forceinline__ void stencil_ld(const Geo& g, const OpK<R>& k, Ld& ld, const C2<R>* __restrict__ Wt,
                                           const C2<R>* __restrict__ Wx, Epi& epi) {
  if (g.march) {
    // The (strip, t) rows of the lattice in strip-major order, split into
    // one contiguous range per warp: ranges differ by at most one row, and a
    // warp restarts its march only where its range crosses into a new strip.
    constexpr int wpb = kBlock / 32;
    const long long rows = (long long)(g.nx >> 5) * g.nt;
    const long long nw = (long long)gridDim.x * wpb;
    const long long gw = (long long)blockIdx.x * wpb + (threadIdx.x >> 5);
    long long r = rows * gw / nw;
    const long long r1 = rows * (gw + 1) / nw;
    while (r < r1) {
      const int xw = (int)(r / g.nt);
      const int ta = (int)(r - (long long)xw * g.nt);
      const int tb = (r1 - r < (long long)(g.nt - ta)) ? ta + (int)(r1 - r) : g.nt;
      march_segment<R, DAG, MU0, UNIT>(g, k, ld, Wt, Wx, xw, ta, tb, epi);
      r += tb - ta;
    }
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

// Blocks of work of a stencil kernel (march: at least kMarchT rows per warp).
inline int stencil_work(const Geo& g) {
  return g.march ? ((g.nx >> 5) * ((g.nt + kMarchT - 1) / kMarchT) + kBlock / 32 - 1) / (kBlock / 32) : nblocks(g.V);
}

}  // namespace tg
