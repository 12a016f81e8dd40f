// tg_fused.cuh -- M^dagger M in one column march (FP32), for the
// single-reduction CG of tg_pcg.cu.
//
// A warp owns 32 consecutive columns x0 .. x0+31 and a range of rows ta .. tb-1
// (for_warp_rows).  It computes u = M v one row ahead of w = M^dagger u, so
// neither u nor a grid barrier between the two operators is needed:
//   * rows: u at rows ta-1 and tb (one above and one below the range) is
//     recomputed by this warp, from v at rows ta-2 .. tb+1;
//   * columns: u at the two columns beside the warp (x0-1 and x0+32), which
//     w at the warp's edge lanes needs, is recomputed once per kMarchT rows by
//     eight lanes (four rows on each side), one site each.
// Every recomputed u is the same dslash_vals call on the same operands as the
// owning warp's, so it equals the owner's value bit for bit.
//
// The vector v the operator acts on is produced by a loader:
//   ld.val(i)  v at site i (halo and edge sites);
//   ld.own(i)  the loader's operand at one of this warp's sites (.v is v; the
//              other fields are what the epilogue needs there).
// epi(s, w(s), u(s), own operand(s)) consumes every site of the range.
#pragma once

#include "tg_stencil.cuh"

namespace tg {

template <bool MU0, class Ld, class Epi>
__device__ __forceinline__ void march_mdagm(const Geo& g, const OpK<float>& km, const OpK<float>& kd, const Ld& ld,
                                            const float2* __restrict__ Wt, const float2* __restrict__ Wx, int xw,
                                            int ta, int tb, Epi& epi) {
  using Op = typename Ld::Op;
  const int nt = g.nt, nx = g.nx;
  const int lane = threadIdx.x & 31;
  const int x0 = xw << 5;
  const int x = x0 + lane;
  const int xle = (x0 == 0) ? nx - 1 : x0 - 1;    // column left of the warp
  const int xre = (x0 + 32 == nx) ? 0 : x0 + 32;  // column right of the warp
  auto wrap = [nt](int t) { return t < 0 ? t + nt : (t >= nt ? t - nt : t); };
  const float2 zero = make_float2(0.f, 0.f);

  // u = M v at one site (t, c), from loads: the halo columns
  auto u_at = [&](int t, int c) -> float2 {
    const int tp = wrap(t + 1), tm = wrap(t - 1);
    const int cp = (c + 1 == nx) ? 0 : c + 1, cm = (c == 0) ? nx - 1 : c - 1;
    const int s = t * nx + c;
    return dslash_vals<float, 0, MU0>(km, ld.val(s), ld.val(tp * nx + c), ld.val(tm * nx + c), ld.val(t * nx + cp),
                                      ld.val(t * nx + cm), Wt[s], Wt[tm * nx + c], Wx[s], Wx[t * nx + cm]);
  };
  // u = M v on one row of the warp: vc = v(t), vu = v(t+1), vd = v(t-1); the
  // operand beyond the warp's edge pe (lanes 0 and 31) and Wx(t, x0-1) we (lane 0)
  auto u_row = [&](float2 vc, float2 vu, float2 vd, float2 wt, float2 wtd, float2 wx, float2 pe, float2 we) {
    float2 pr = shfl_down1<float>(vc), pl = shfl_up1<float>(vc), wl = shfl_up1<float>(wx);
    if (lane == 31) pr = pe;
    if (lane == 0) {
      pl = pe;
      wl = we;
    }
    return dslash_vals<float, 0, MU0>(km, vc, vu, vd, pr, pl, wt, wtd, wx, wl);
  };
  // w = M^dag u on one row: uc = u(t), uu = u(t+1), ud = u(t-1); ue = u beyond
  // the edge (lanes 0 and 31), we = Wx(t, x0-1) (lane 0)
  auto w_row = [&](float2 uc, float2 uu, float2 ud, float2 wt, float2 wtd, float2 wx, float2 ue, float2 we) {
    float2 ur = shfl_down1<float>(uc), ul = shfl_up1<float>(uc), wl = shfl_up1<float>(wx);
    if (lane == 31) ur = ue;
    if (lane == 0) {
      ul = ue;
      wl = we;
    }
    return dslash_vals<float, 1, MU0>(kd, uc, uu, ud, ur, ul, wt, wtd, wx, wl);
  };
  const int xe = (lane == 31) ? xre : xle;  // the edge column lanes 0 and 31 use

  // ---- prologue: u(ta-1), u(ta) ----
  const int tm1 = wrap(ta - 1), tm2 = wrap(ta - 2), tp1 = wrap(ta + 1);
  const float2 v_mm = ld.val(tm2 * nx + x);
  const float2 v_m = ld.val(tm1 * nx + x);
  Op o_c = ld.own(ta * nx + x);
  Op o_n = ld.own(tp1 * nx + x);
  const float2 wt_mm = Wt[tm2 * nx + x];
  float2 wt_m = Wt[tm1 * nx + x], wt_c = Wt[ta * nx + x];
  const float2 wx_m = Wx[tm1 * nx + x];
  float2 wx_c = Wx[ta * nx + x];
  float2 pe_m = zero, pe_c = zero, we_m = zero, we_c = zero;
  if (lane == 0 || lane == 31) {
    pe_m = ld.val(tm1 * nx + xe);
    pe_c = ld.val(ta * nx + xe);
    we_m = Wx[tm1 * nx + xle];
    we_c = Wx[ta * nx + xle];
  }
  float2 u_m = u_row(v_m, o_c.v, v_mm, wt_m, wt_mm, wx_m, pe_m, we_m);
  float2 u_c = u_row(o_c.v, o_n.v, v_m, wt_c, wt_m, wx_c, pe_c, we_c);

  // ---- chunks of kMarchT output rows ----
  int t = ta;
  for (; t + kMarchT <= tb; t += kMarchT) {
    Op on[kMarchT];
    float2 wtn[kMarchT], wxn[kMarchT];
#pragma unroll
    for (int i = 0; i < kMarchT; i++) {
      const int r1 = wrap(t + 1 + i);
      on[i] = ld.own(wrap(t + 2 + i) * nx + x);
      wtn[i] = Wt[r1 * nx + x];
      wxn[i] = Wx[r1 * nx + x];
    }
    // lanes i < kMarchT: the left edge of row t+i; lanes kMarchT+i: the right edge
    float2 er = zero, ewl = zero, eu = zero;
    if (lane < 2 * kMarchT) {
      const int i = lane & (kMarchT - 1);
      const int c = (lane < kMarchT) ? xle : xre;
      er = ld.val(wrap(t + 1 + i) * nx + c);   // v(t+1+i) beyond the edge, for u(t+1+i)
      if (lane < kMarchT) ewl = Wx[wrap(t + 1 + i) * nx + xle];
      eu = u_at(t + i, c);                     // u(t+i) beyond the edge, for w(t+i)
    }
#pragma unroll
    for (int i = 0; i < kMarchT; i++) {
      const int src = (lane == 31) ? kMarchT + i : i;
      const float2 pe = shfl_c2<float>(er, src);
      const float2 we = shfl_c2<float>(ewl, i);
      const float2 ue = shfl_c2<float>(eu, src);
      const float2 u_n = u_row(o_n.v, on[i].v, o_c.v, wtn[i], wt_c, wxn[i], pe, we);
      const float2 w = w_row(u_c, u_n, u_m, wt_c, wt_m, wx_c, ue, we_c);
      epi((t + i) * nx + x, w, u_c, o_c);
      u_m = u_c;
      u_c = u_n;
      o_c = o_n;
      o_n = on[i];
      wt_m = wt_c;
      wt_c = wtn[i];
      wx_c = wxn[i];
      we_c = we;
    }
  }
  // ---- the last rows of the range, one at a time ----
  for (; t < tb; t++) {
    const int r1 = wrap(t + 1);
    const Op onn = ld.own(wrap(t + 2) * nx + x);
    const float2 wtn = Wt[r1 * nx + x], wxn = Wx[r1 * nx + x];
    float2 pe = zero, we = zero, ue = zero;
    if (lane == 0 || lane == 31) {
      pe = ld.val(r1 * nx + xe);
      we = Wx[r1 * nx + xle];
      ue = u_at(t, xe);
    }
    const float2 u_n = u_row(o_n.v, onn.v, o_c.v, wtn, wt_c, wxn, pe, we);
    const float2 w = w_row(u_c, u_n, u_m, wt_c, wt_m, wx_c, ue, we_c);
    epi(t * nx + x, w, u_c, o_c);
    u_m = u_c;
    u_c = u_n;
    o_c = o_n;
    o_n = onn;
    wt_m = wt_c;
    wt_c = wtn;
    wx_c = wxn;
    we_c = we;
  }
}

// M^dagger M over every site of the lattice (column-march lattices only: nx a
// multiple of 32, nt of kMarchT), the rows split over the grid's warps.
template <bool MU0, class Ld, class Epi>
__device__ __forceinline__ void stencil_mdagm(const Geo& g, const OpK<float>& km, const OpK<float>& kd, const Ld& ld,
                                              const float2* __restrict__ Wt, const float2* __restrict__ Wx, Epi& epi) {
  for_warp_rows(g, [&](int xw, int ta, int tb) { march_mdagm<MU0>(g, km, kd, ld, Wt, Wx, xw, ta, tb, epi); });
}

}  // namespace tg
