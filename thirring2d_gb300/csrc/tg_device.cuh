// tg_device.cuh -- device functions shared by the single-lattice kernels
// (tg_kernels.cu) and the batched-chain kernel (tg_batch.cu): link
// coefficients, the staggered operator at one site, the force at one site, and
// the Philox generator.  One implementation, so both paths compute the same
// numbers for the same inputs.
#pragma once

#include <math.h>

#include "tg_launch.h"

namespace tg {

// ---------------------------------------------------------------------------
// Link coefficients  W_mu(s) = 0.5 * eta_mu(s) * bc_mu(s) * (cos A, sin A)
// eta_t(x) = (-1)^x, eta_x = 1 (hmc.c:914-921); bc_mu applies on the link that
// leaves the last slice (hmc.c:143-148, 165-170).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void link_vals(const Geo& g, int bc_t, int bc_x, int s, double2 a, double2& wt,
                                          double2& wx) {
  int t, x;
  site_tx(g, s, t, x);
  double ft = 0.5 * ((x & 1) ? -1.0 : 1.0) * ((t == g.nt - 1) ? (double)bc_t : 1.0);
  double fx = 0.5 * ((x == g.nx - 1) ? (double)bc_x : 1.0);
  double st, ct, sx, cx;
  sincos(a.x, &st, &ct);
  sincos(a.y, &sx, &cx);
  wt = make_double2(ft * ct, ft * st);
  wx = make_double2(fx * cx, fx * sx);
}

__device__ __forceinline__ void write_links(const Geo& g, int bc_t, int bc_x, int s, double2 a, double2* Wt,
                                            double2* Wx, float2* Wt32, float2* Wx32) {
  double2 wt, wx;
  link_vals(g, bc_t, bc_x, s, a, wt, wx);
  Wt[s] = wt;
  Wx[s] = wx;
  Wt32[s] = make_float2((float)wt.x, (float)wt.y);
  Wx32[s] = make_float2((float)wx.x, (float)wx.y);
}

// ... and W / m for the unit-mass operator M / m = 1 + D / m when o.Wt1 is set
__device__ __forceinline__ void write_links(const Geo& g, int bc_t, int bc_x, int s, double2 a, const LinkOut& o) {
  double2 wt, wx;
  link_vals(g, bc_t, bc_x, s, a, wt, wx);
  o.Wt[s] = wt;
  o.Wx[s] = wx;
  o.Wt32[s] = make_float2((float)wt.x, (float)wt.y);
  o.Wx32[s] = make_float2((float)wx.x, (float)wx.y);
  if (o.Wt1 != nullptr) {
    o.Wt1[s] = make_double2(wt.x * o.inv_m, wt.y * o.inv_m);
    o.Wx1[s] = make_double2(wx.x * o.inv_m, wx.y * o.inv_m);
  }
}

// ---------------------------------------------------------------------------
// The staggered operator at one site: hmc.c:132-183 for M (DAG = 0) and the
// true adjoint M^dagger = m - D(-mu) (DAG = 1).  MU0 drops the e^{+-mu}
// factors (mu = 0): 18 FMA/MUL per site instead of 22.  UNIT applies
// M / m = 1 + D / m instead (the links passed in are then W / m): the mass
// product goes, 16 FMA per site.
// ---------------------------------------------------------------------------
template <typename R, int DAG, bool MU0, bool UNIT = false>
__device__ __forceinline__ C2<R> dslash_vals(const OpK<R>& k, C2<R> pc, C2<R> ptu, C2<R> ptd, C2<R> pxu, C2<R> pxd,
                                             C2<R> wt, C2<R> wtd, C2<R> wx, C2<R> wxd) {
  // pc = in(s); ptu/ptd = in(s+t)/in(s-t); pxu/pxd = in(s+x)/in(s-x);
  // wt = Wt(s), wtd = Wt(s-t), wx = Wx(s), wxd = Wx(s-x)
  C2<R> o = UNIT ? pc : mk<R>(k.m * pc.x, k.m * pc.y);
  if (MU0) {
    if (DAG == 0) {
      cmac<R>(o, wt, ptu);
      cmsc<R>(o, wtd, ptd);
    } else {
      cnmac<R>(o, wt, ptu);
      cjmac<R>(o, wtd, ptd);
    }
  } else {
    C2<R> ft = cmul<R>(wt, ptu);
    C2<R> bt = cjmul<R>(wtd, ptd);
    o.x = fma(k.cf, ft.x, o.x);
    o.y = fma(k.cf, ft.y, o.y);
    o.x = fma(k.cb, bt.x, o.x);
    o.y = fma(k.cb, bt.y, o.y);
  }
  if (DAG == 0) {
    cmac<R>(o, wx, pxu);
    cmsc<R>(o, wxd, pxd);
  } else {
    cnmac<R>(o, wx, pxu);
    cjmac<R>(o, wxd, pxd);
  }
  return o;
}

template <typename R, int DAG, bool MU0>
__device__ __forceinline__ C2<R> dslash_site(const OpK<R>& k, const C2<R>* __restrict__ in,
                                             const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx, int s,
                                             const Nbr& n) {
  return dslash_vals<R, DAG, MU0>(k, in[s], in[n.tp], in[n.tm], in[n.xp], in[n.xm], Wt[s], Wt[n.tm], Wx[s],
                                  Wx[n.xm]);
}

template <typename R, int DAG, bool MU0>
__device__ __forceinline__ C2<R> dslash_at(const Geo& g, const OpK<R>& k, const C2<R>* __restrict__ in,
                                           const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx, int s) {
  int t, x;
  site_tx(g, s, t, x);
  return dslash_site<R, DAG, MU0>(k, in, Wt, Wx, s, neighbours(g, s, t, x));
}

template <typename R> __device__ __forceinline__ C2<R> shfl_down1(C2<R> v) {
  return mk<R>(__shfl_down_sync(0xffffffffu, v.x, 1), __shfl_down_sync(0xffffffffu, v.y, 1));
}
template <typename R> __device__ __forceinline__ C2<R> shfl_up1(C2<R> v) {
  return mk<R>(__shfl_up_sync(0xffffffffu, v.x, 1), __shfl_up_sync(0xffffffffu, v.y, 1));
}

// Force pieces at one site (momentum_step, hmc.c:504-661):
//   gauge   (Nf/g) sin A                                           (507-510)
//   pf      2 Im W (e^{mu} conj(Mchi(s)) chi(s+mu) - e^{-mu} conj(chi(s)) Mchi(s+mu))   (517-576)
//   noise   -(e^{mu} - e^{-mu}) Im W conj(n(s)) n(s+t), t links only  (608-661)
struct ForcePieces {
  double2 g, pf, md;
};

// The gauge force's sin A comes from the link coefficient the same gauge step
// wrote: W = f e^{iA} with f = +-1/2, so sin A = Im W / f exactly (f and 1/f
// are powers of two).  A link with f = 0 (open boundary) takes sin A itself.
__device__ __forceinline__ ForcePieces force_site(const Geo& g, int bc_t, int bc_x, double ep, double em,
                                                  const double2* A, const double2* Wt, const double2* Wx,
                                                  const double2* chi, const double2* Mchi, const double2* noise,
                                                  int s) {
  int t, x;
  site_tx(g, s, t, x);
  Nbr n = neighbours(g, s, t, x);
  ForcePieces f;
  const double bt = (t == g.nt - 1) ? (double)bc_t : 1.0;
  const double bx = (x == g.nx - 1) ? (double)bc_x : 1.0;
  const double inv_ft = ((x & 1) ? -2.0 : 2.0) * bt, inv_fx = 2.0 * bx;
  f.g.x = (bt != 0.0) ? Wt[s].y * inv_ft : sin(A[s].x);
  f.g.y = (bx != 0.0) ? Wx[s].y * inv_fx : sin(A[s].y);
  f.pf = make_double2(0, 0);
  f.md = make_double2(0, 0);
  if (chi != nullptr) {
    double2 c0 = chi[s], m0 = Mchi[s];
    double2 ct = chi[n.tp], mt = Mchi[n.tp];
    double2 cx = chi[n.xp], mx = Mchi[n.xp];
    // e1*conj(m0)*c_next - e2*conj(c0)*m_next
    double2 q1 = cjmul<double>(m0, ct), q2 = cjmul<double>(c0, mt);
    double2 qt = make_double2(ep * q1.x - em * q2.x, ep * q1.y - em * q2.y);
    double2 r1 = cjmul<double>(m0, cx), r2 = cjmul<double>(c0, mx);
    double2 qx = make_double2(r1.x - r2.x, r1.y - r2.y);
    double2 wt = Wt[s], wx = Wx[s];
    f.pf.x = 2.0 * fma(wt.x, qt.y, wt.y * qt.x);
    f.pf.y = 2.0 * fma(wx.x, qx.y, wx.y * qx.x);
  }
  if (noise != nullptr) {
    double d = ep - em;
    double2 q = cjmul<double>(noise[s], noise[n.tp]);
    double2 wt = Wt[s];
    f.md.x = -d * fma(wt.x, q.y, wt.y * q.x);
  }
  return f;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter = (site,
// stream, trajectory lo, trajectory hi), key = seed.  Each draw gives two
// 53-bit uniforms in (0,1) -> one Box-Muller pair.
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
  for (int i = 0; i < 10; i++) {
    unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ double u53(unsigned hi, unsigned lo) {
  // ((hi:lo) >> 11 + 0.5) * 2^-53, strictly inside (0,1)
  unsigned long long v = ((unsigned long long)hi << 21) ^ (lo >> 11);
  return ((double)v + 0.5) * 1.1102230246251565e-16;
}

__device__ __forceinline__ double2 philox_gauss_pair(unsigned long long seed, unsigned long long tr, unsigned site,
                                                     unsigned stream_id) {
  uint4 r = philox4x32(make_uint4(site, stream_id, (unsigned)tr, (unsigned)(tr >> 32)),
                       make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
  double u1 = u53(r.x, r.y), u2 = u53(r.z, r.w);
  double rad = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  return make_double2(rad * cs, rad * sn);
}

__device__ __forceinline__ double philox_uniform1(unsigned long long seed, unsigned long long tr, unsigned stream_id) {
  uint4 r = philox4x32(make_uint4(0xffffffffu, stream_id, (unsigned)tr, (unsigned)(tr >> 32)),
                       make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
  return u53(r.x, r.y);
}

}  // namespace tg
