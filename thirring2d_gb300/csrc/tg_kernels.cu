// tg_kernels.cu -- sm_103a kernels of the Thirring2D HMC hot path.
//
// All kernels are one-thread-per-site over the t-major site index, 256-thread
// blocks, coalesced double2/float2 loads.  Stencil neighbours along x are in
// the same or adjacent warps and along t one row (nx sites) away, so each
// operand is fetched from DRAM once and re-read from L1/L2.  Reductions are
// deterministic (fixed shuffle tree per block, partials summed in index order
// by the last block), so results do not depend on block scheduling.
#include <math.h>

#include "tg_launch.h"

namespace tg {

// ---------------------------------------------------------------------------
// Link coefficients  W_mu(s) = 0.5 * eta_mu(s) * bc_mu(s) * (cos A, sin A)
// eta_t(x) = (-1)^x, eta_x = 1 (hmc.c:914-921); bc_mu applies on the link that
// leaves the last slice (hmc.c:143-148, 165-170).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void write_links(const Geo& g, int bc_t, int bc_x, int s, double2 a, double2* Wt,
                                            double2* Wx, float2* Wt32, float2* Wx32) {
  int t, x;
  site_tx(g, s, t, x);
  double ft = 0.5 * ((x & 1) ? -1.0 : 1.0) * ((t == g.nt - 1) ? (double)bc_t : 1.0);
  double fx = 0.5 * ((x == g.nx - 1) ? (double)bc_x : 1.0);
  double st, ct, sx, cx;
  sincos(a.x, &st, &ct);
  sincos(a.y, &sx, &cx);
  double2 wt = make_double2(ft * ct, ft * st);
  double2 wx = make_double2(fx * cx, fx * sx);
  Wt[s] = wt;
  Wx[s] = wx;
  Wt32[s] = make_float2((float)wt.x, (float)wt.y);
  Wx32[s] = make_float2((float)wx.x, (float)wx.y);
}

__global__ void __launch_bounds__(kBlock) k_link_phase(Geo g, int bc_t, int bc_x, const double2* __restrict__ A,
                                                       double2* Wt, double2* Wx, float2* Wt32, float2* Wx32) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  write_links(g, bc_t, bc_x, s, A[s], Wt, Wx, Wt32, Wx32);
}

// gauge_step (hmc.c:97-101) applied nadd times: A += c*p with c = 2*eps.
__global__ void __launch_bounds__(kBlock) k_gauge_step(Geo g, int bc_t, int bc_x, double2* A,
                                                       const double2* __restrict__ mom, double c, int nadd,
                                                       double2* Wt, double2* Wx, float2* Wt32, float2* Wx32) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  double2 a = A[s];
  double2 p = mom[s];
  for (int k = 0; k < nadd; k++) {  // product then sum, two roundings, as the host code of hmc.c:99
    a.x = __dadd_rn(a.x, __dmul_rn(c, p.x));
    a.y = __dadd_rn(a.y, __dmul_rn(c, p.y));
  }
  A[s] = a;
  write_links(g, bc_t, bc_x, s, a, Wt, Wx, Wt32, Wx32);
}

void link_phase(cudaStream_t s, const Geo& g, int bc_t, int bc_x, const double2* A, double2* Wt, double2* Wx,
                float2* Wt32, float2* Wx32) {
  k_link_phase<<<nblocks(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, A, Wt, Wx, Wt32, Wx32);
}
void gauge_step(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double2* A, const double2* mom, double c,
                int nadd, double2* Wt, double2* Wx, float2* Wt32, float2* Wx32) {
  k_gauge_step<<<nblocks(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, A, mom, c, nadd, Wt, Wx, Wt32, Wx32);
}

// ---------------------------------------------------------------------------
// The staggered operator at one site (hmc.c:132-183 for M; the true adjoint
// for M^dagger through the OpK constants).
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ C2<R> dslash_site(const OpK<R>& k, const C2<R>* __restrict__ in,
                                             const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx, int s,
                                             const Nbr& n) {
  C2<R> v = in[s];
  C2<R> ft = cmul<R>(Wt[s], in[n.tp]);
  C2<R> bt = cjmul<R>(Wt[n.tm], in[n.tm]);
  C2<R> hx = mk<R>(0, 0);
  cmac<R>(hx, Wx[s], in[n.xp]);
  cmsc<R>(hx, Wx[n.xm], in[n.xm]);
  C2<R> o;
  o.x = k.m * v.x;
  o.y = k.m * v.y;
  o.x = fma(k.cf, ft.x, o.x);
  o.y = fma(k.cf, ft.y, o.y);
  o.x = fma(k.cb, bt.x, o.x);
  o.y = fma(k.cb, bt.y, o.y);
  o.x = fma(k.cx, hx.x, o.x);
  o.y = fma(k.cx, hx.y, o.y);
  return o;
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_dslash(Geo g, OpK<R> k, const C2<R>* __restrict__ in,
                                                   C2<R>* __restrict__ out, const C2<R>* __restrict__ Wt,
                                                   const C2<R>* __restrict__ Wx) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  int t, x;
  site_tx(g, s, t, x);
  out[s] = dslash_site<R>(k, in, Wt, Wx, s, neighbours(g, s, t, x));
}

void dslash64(cudaStream_t s, const Geo& g, const OpK<double>& k, const double2* in, double2* out,
              const double2* Wt, const double2* Wx) {
  k_dslash<double><<<nblocks(g.V), kBlock, 0, s>>>(g, k, in, out, Wt, Wx);
}
void dslash32(cudaStream_t s, const Geo& g, const OpK<float>& k, const float2* in, float2* out, const float2* Wt,
              const float2* Wx) {
  k_dslash<float><<<nblocks(g.V), kBlock, 0, s>>>(g, k, in, out, Wt, Wx);
}

// ---------------------------------------------------------------------------
// CG on M^dagger M (fmdm_invert_cg, hmc.c:341-404), one iteration =
//   K1: Mp = M p,  pAp = |Mp|^2,            alpha = rr / pAp
//   K2: x += alpha p, r -= alpha M^dag Mp,  rr' = |r|^2, beta = rr'/rr, tests
//   K3: p = r + beta p
// pAp = <p, M^dag M p> is taken as |Mp|^2 (same value, always >= 0).  The
// scalar recurrences run in the last block of K1/K2, so the host never waits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cg_finish(CgState* st, CgLog* log, int status, Cond c) {
  st->status = status;
  st->done = 1;
  if (log != nullptr && st->log_index >= 0) {
    CgLog& l = log[st->log_index];
    l.iter = st->iter;
    l.status = status;
    l.n_ru = st->n_ru;
    l.rr = st->rr;
    l.rr0 = st->rr0;
  }
  if (c.use) cudaGraphSetConditional(c.loop, 0);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_cg_init(Geo g, const double2* __restrict__ b, double2* x, C2<R>* r,
                                                    C2<R>* p, C2<R>* xs, double rel_tol, double abs_tol2,
                                                    int maxiter, int ru_interval, int log_index, CgState* st,
                                                    CgLog* log, Red red, Cond c) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  double v = 0;
  if (s < g.V) {
    double2 bb = b[s];
    x[s] = make_double2(0.0, 0.0);
    C2<R> rb = mk<R>((R)bb.x, (R)bb.y);
    r[s] = rb;
    p[s] = rb;
    if (xs != nullptr) xs[s] = mk<R>(0, 0);
    v = bb.x * bb.x + bb.y * bb.y;
  }
  double tot;
  if (grid_sum<kBlock>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) {
    double stop = abs_tol2;
    if (rel_tol > 0 && rel_tol * rel_tol * tot > stop) stop = rel_tol * rel_tol * tot;
    st->rr = tot;
    st->rr0 = tot;
    st->rr_true = tot;
    st->stop = stop;
    st->alpha = 0;
    st->beta = 0;
    st->iter = 0;
    st->maxiter = maxiter;
    st->status = 0;
    st->since_ru = 0;
    st->ru_interval = ru_interval;
    st->n_ru = 0;
    st->need_ru = 0;
    st->restart = 0;
    st->log_index = log_index;
    // b = 0 or already below the stop (hmc.c:359-361), or NaN: no iterations
    int done = !(tot >= stop) || tot == 0.0;
    st->done = 0;
    if (done) cg_finish(st, log, isnan(tot) ? TG_E_NAN : TG_OK, c);
    else if (c.use) cudaGraphSetConditional(c.loop, 1u);
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_cg1(Geo g, OpK<R> k, const C2<R>* __restrict__ p, C2<R>* __restrict__ Mp,
                                                const C2<R>* __restrict__ Wt, const C2<R>* __restrict__ Wx,
                                                CgState* st, Red red) {
  if (st->done) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  double v = 0;
  if (s < g.V) {
    int t, x;
    site_tx(g, s, t, x);
    C2<R> o = dslash_site<R>(k, p, Wt, Wx, s, neighbours(g, s, t, x));
    Mp[s] = o;
    v = (double)o.x * (double)o.x + (double)o.y * (double)o.y;
  }
  double tot;
  if (grid_sum<kBlock>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) {
    st->alpha = st->rr / tot;
    st->need_ru = 0;   // the previous iteration's reliable-update kernels have all run
    st->restart = 0;
  }
}

// FP64: convergence tested on the recursive residual, as hmc.c:381.
__global__ void __launch_bounds__(kBlock) k_cg2_64(Geo g, OpK<double> k, const double2* __restrict__ Mp,
                                                   const double2* __restrict__ p, double2* __restrict__ x,
                                                   double2* __restrict__ r, const double2* __restrict__ Wt,
                                                   const double2* __restrict__ Wx, CgState* st, CgLog* log,
                                                   Red red, Cond c) {
  if (st->done) return;
  const double a = st->alpha;
  int s = blockIdx.x * kBlock + threadIdx.x;
  double v = 0;
  if (s < g.V) {
    int t, xx;
    site_tx(g, s, t, xx);
    double2 ap = dslash_site<double>(k, Mp, Wt, Wx, s, neighbours(g, s, t, xx));
    double2 xv = x[s], pv = p[s], rv = r[s];
    xv.x += a * pv.x;
    xv.y += a * pv.y;
    rv.x -= a * ap.x;
    rv.y -= a * ap.y;
    x[s] = xv;
    r[s] = rv;
    v = rv.x * rv.x + rv.y * rv.y;
  }
  double rn;
  if (grid_sum<kBlock>(v, red.partials, red.counter, &rn) && threadIdx.x == 0) {
    st->iter += 1;
    double rr_old = st->rr;
    st->rr = rn;
    st->beta = rn / rr_old;
    if (isnan(rn)) cg_finish(st, log, TG_E_NAN, c);
    else if (rn < st->stop) cg_finish(st, log, TG_OK, c);
    else if (rn / st->rr0 > 1e10) cg_finish(st, log, TG_E_DIVERGED, c);
    else if (st->iter >= st->maxiter) cg_finish(st, log, TG_E_NOCONV, c);
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_cg3(int n, const C2<R>* __restrict__ r, C2<R>* __restrict__ p,
                                                const CgState* st) {
  if (st->done) return;
  const R b = (R)st->beta;
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= n) return;
  C2<R> rv = r[s], pv = p[s];
  p[s] = mk<R>(rv.x + b * pv.x, rv.y + b * pv.y);
}

void cg64_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufs64& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int log_index, Cond c) {
  k_cg_init<double><<<nblocks(g.V), kBlock, 0, s>>>(g, b, x, w.r, w.p, nullptr, rel_tol, abs_tol2, maxiter, 0,
                                                    log_index, st, log, red, c);
}

void cg64_iter(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
               double2* x, const CgBufs64& w, CgState* st, CgLog* log, const Red& red, Cond c) {
  int nb = nblocks(g.V);
  k_cg1<double><<<nb, kBlock, 0, s>>>(g, km, w.p, w.Mp, L.Wt, L.Wx, st, red);
  k_cg2_64<<<nb, kBlock, 0, s>>>(g, kd, w.Mp, w.p, x, w.r, L.Wt, L.Wx, st, log, red, c);
  k_cg3<double><<<nb, kBlock, 0, s>>>(g.V, w.r, w.p, st);
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 vectors and links, FP64 scalar recurrences.  x
// accumulates in FP64 at each reliable update (every ru_interval iterations,
// when the FP32 residual reaches the target, or at the iteration cap), which
// recomputes r = b - M^dag M x in FP64 and restarts the FP32 residual from it.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_cgmx2(Geo g, OpK<float> k, const float2* __restrict__ Mp,
                                                  const float2* __restrict__ p, float2* __restrict__ xs,
                                                  float2* __restrict__ r, const float2* __restrict__ Wt,
                                                  const float2* __restrict__ Wx, CgState* st, Red red, Cond c) {
  if (st->done) return;
  const float a = (float)st->alpha;
  int s = blockIdx.x * kBlock + threadIdx.x;
  double v = 0;
  if (s < g.V) {
    int t, xx;
    site_tx(g, s, t, xx);
    float2 ap = dslash_site<float>(k, Mp, Wt, Wx, s, neighbours(g, s, t, xx));
    float2 xv = xs[s], pv = p[s], rv = r[s];
    xv.x = fmaf(a, pv.x, xv.x);
    xv.y = fmaf(a, pv.y, xv.y);
    rv.x = fmaf(-a, ap.x, rv.x);
    rv.y = fmaf(-a, ap.y, rv.y);
    xs[s] = xv;
    r[s] = rv;
    v = (double)rv.x * rv.x + (double)rv.y * rv.y;
  }
  double rn;
  if (grid_sum<kBlock>(v, red.partials, red.counter, &rn) && threadIdx.x == 0) {
    st->iter += 1;
    st->since_ru += 1;
    double rr_old = st->rr;
    st->rr = rn;
    st->beta = rn / rr_old;
    int need = st->since_ru >= st->ru_interval || rn < st->stop || rn < kRuDrop * st->rr_true ||
               st->iter >= st->maxiter || rn / st->rr0 > 1e10 || isnan(rn);
    st->need_ru = need;
    if (c.use) cudaGraphSetConditional(c.ru, need ? 1u : 0u);
  }
}

// reliable update 1: x += xs, xs = 0
__global__ void __launch_bounds__(kBlock) k_ru1(int n, double2* x, float2* xs, const CgState* st) {
  if (!st->need_ru || st->done) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= n) return;
  float2 d = xs[s];
  double2 v = x[s];
  v.x += (double)d.x;
  v.y += (double)d.y;
  x[s] = v;
  xs[s] = make_float2(0.f, 0.f);
}

// reliable update 2: tmp = M x (FP64)
__global__ void __launch_bounds__(kBlock) k_ru2(Geo g, OpK<double> k, const double2* __restrict__ x,
                                                double2* __restrict__ tmp, const double2* __restrict__ Wt,
                                                const double2* __restrict__ Wx, const CgState* st) {
  if (!st->need_ru || st->done) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  int t, xx;
  site_tx(g, s, t, xx);
  tmp[s] = dslash_site<double>(k, x, Wt, Wx, s, neighbours(g, s, t, xx));
}

// reliable update 3: r = b - M^dag tmp (FP64), rs = (float) r, decide
__global__ void __launch_bounds__(kBlock) k_ru3(Geo g, OpK<double> k, const double2* __restrict__ b,
                                                const double2* __restrict__ tmp, float2* __restrict__ rs,
                                                const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                CgState* st, CgLog* log, Red red, Cond c) {
  if (!st->need_ru || st->done) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  double v = 0;
  if (s < g.V) {
    int t, xx;
    site_tx(g, s, t, xx);
    double2 ap = dslash_site<double>(k, tmp, Wt, Wx, s, neighbours(g, s, t, xx));
    double2 bb = b[s];
    double2 rv = make_double2(bb.x - ap.x, bb.y - ap.y);
    rs[s] = make_float2((float)rv.x, (float)rv.y);
    v = rv.x * rv.x + rv.y * rv.y;
  }
  double rt;
  if (grid_sum<kBlock>(v, red.partials, red.counter, &rt) && threadIdx.x == 0) {
    st->restart = rt > kRuRestart * st->rr;  // recursive residual was far too optimistic
    st->rr_true = rt;
    st->rr = rt;
    st->since_ru = 0;
    st->n_ru += 1;
    if (isnan(rt)) cg_finish(st, log, TG_E_NAN, c);
    else if (rt < st->stop) cg_finish(st, log, TG_OK, c);
    else if (rt / st->rr0 > 1e10) cg_finish(st, log, TG_E_DIVERGED, c);
    else if (st->iter >= st->maxiter) cg_finish(st, log, TG_E_NOCONV, c);
  }
}

// reliable update 4: restart the search direction from the new residual
__global__ void __launch_bounds__(kBlock) k_ru4(int n, const float2* __restrict__ rs, float2* __restrict__ ps,
                                                const CgState* st) {
  if (!st->need_ru || !st->restart || st->done) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s < n) ps[s] = rs[s];
}

void cgmx_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufsMixed& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int ru_interval,
               int log_index, Cond c) {
  k_cg_init<float><<<nblocks(g.V), kBlock, 0, s>>>(g, b, x, w.rs, w.ps, w.xs, rel_tol, abs_tol2, maxiter,
                                                   ru_interval, log_index, st, log, red, c);
}

void cgmx_iter(cudaStream_t s, const Geo& g, const OpK<float>& km, const OpK<float>& kd, const Links& L,
               const CgBufsMixed& w, CgState* st, const Red& red, Cond c) {
  int nb = nblocks(g.V);
  k_cg1<float><<<nb, kBlock, 0, s>>>(g, km, w.ps, w.Mps, L.Wt32, L.Wx32, st, red);
  k_cgmx2<<<nb, kBlock, 0, s>>>(g, kd, w.Mps, w.ps, w.xs, w.rs, L.Wt32, L.Wx32, st, red, c);
  k_cg3<float><<<nb, kBlock, 0, s>>>(g.V, w.rs, w.ps, st);
}

void cgmx_reliable(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
                   const double2* b, double2* x, const CgBufsMixed& w, CgState* st, CgLog* log, const Red& red,
                   Cond c) {
  int nb = nblocks(g.V);
  k_ru1<<<nb, kBlock, 0, s>>>(g.V, x, w.xs, st);
  k_ru2<<<nb, kBlock, 0, s>>>(g, km, x, w.tmp64, L.Wt, L.Wx, st);
  k_ru3<<<nb, kBlock, 0, s>>>(g, kd, b, w.tmp64, w.rs, L.Wt, L.Wx, st, log, red, c);
  k_ru4<<<nb, kBlock, 0, s>>>(g.V, w.rs, w.ps, st);
}

// ---------------------------------------------------------------------------
// Reductions for the Hamiltonian (hmc.c:73-79, 428, 451-463, 467-479, 493, 723)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_norm2(int n, const double2* __restrict__ v, double* dst, int acc,
                                                  Red red) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  double a = 0;
  if (s < n) {
    double2 u = v[s];
    a = u.x * u.x + u.y * u.y;
  }
  double tot;
  if (grid_sum<kBlock>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = acc ? *dst + tot : tot;
}

__global__ void __launch_bounds__(kBlock) k_redot(int n, const double2* __restrict__ u, const double2* __restrict__ v,
                                                  double* dst, int acc, Red red) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  double a = 0;
  if (s < n) {
    double2 x = u[s], y = v[s];
    a = x.x * y.x + x.y * y.y;
  }
  double tot;
  if (grid_sum<kBlock>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = acc ? *dst + tot : tot;
}

__global__ void __launch_bounds__(kBlock) k_gauge_action(int n, const double2* __restrict__ A, double fac,
                                                         double* dst, Red red) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  double a = 0;
  if (s < n) {
    double2 v = A[s];
    a = (1. - cos(v.x)) + (1. - cos(v.y));
  }
  double tot;
  if (grid_sum<kBlock>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = fac * tot;
}

__global__ void __launch_bounds__(kBlock) k_md_action(Geo g, OpK<double> k, const double2* __restrict__ nz,
                                                      const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                      double* dst, Red red) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  double a = 0;
  if (s < g.V) {
    int t, x;
    site_tx(g, s, t, x);
    double2 o = dslash_site<double>(k, nz, Wt, Wx, s, neighbours(g, s, t, x));
    double2 v = nz[s];
    a = v.x * o.x + v.y * o.y;
  }
  double tot;
  if (grid_sum<kBlock>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = tot;
}

void norm2(cudaStream_t s, int n, const double2* v, double* dst, int accumulate, const Red& red) {
  k_norm2<<<nblocks(n), kBlock, 0, s>>>(n, v, dst, accumulate, red);
}
void redot(cudaStream_t s, int n, const double2* u, const double2* v, double* dst, int accumulate, const Red& red) {
  k_redot<<<nblocks(n), kBlock, 0, s>>>(n, u, v, dst, accumulate, red);
}
void gauge_action(cudaStream_t s, int n, const double2* A, double fac, double* dst, const Red& red) {
  k_gauge_action<<<nblocks(n), kBlock, 0, s>>>(n, A, fac, dst, red);
}
void md_action(cudaStream_t s, const Geo& g, const OpK<double>& kd, const double2* nz, const double2* Wt,
               const double2* Wx, double* dst, const Red& red) {
  k_md_action<<<nblocks(g.V), kBlock, 0, s>>>(g, kd, nz, Wt, Wx, dst, red);
}

// ---------------------------------------------------------------------------
// Force (momentum_step, hmc.c:504-661), per link:
//   gauge   (Nf/g) sin A                                           (507-510)
//   pf      2 Im W (e^{mu} conj(Mchi(s)) chi(s+mu) - e^{-mu} conj(chi(s)) Mchi(s+mu))   (517-576)
//   noise   -(e^{mu} - e^{-mu}) Im W conj(n(s)) n(s+t), t links only  (608-661)
// with e^{+-mu} on t links only.  The three parts are subtracted from p in
// the reference's order.
// ---------------------------------------------------------------------------
struct ForcePieces {
  double2 g, pf, md;
};

__device__ __forceinline__ ForcePieces force_site(const Geo& g, double ep, double em, const double2* A,
                                                  const double2* Wt, const double2* Wx, const double2* chi,
                                                  const double2* Mchi, const double2* noise, int s) {
  int t, x;
  site_tx(g, s, t, x);
  Nbr n = neighbours(g, s, t, x);
  ForcePieces f;
  double2 a = A[s];
  f.g = make_double2(sin(a.x), sin(a.y));
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

__global__ void __launch_bounds__(kBlock) k_momentum_update(Geo g, double ep, double em, const double2* __restrict__ A,
                                                            const double2* __restrict__ Wt,
                                                            const double2* __restrict__ Wx,
                                                            const double2* __restrict__ chi,
                                                            const double2* __restrict__ Mchi,
                                                            const double2* __restrict__ noise, double2* mom,
                                                            double eps, double gfac, int flags) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  ForcePieces f = force_site(g, ep, em, A, Wt, Wx, chi, Mchi, (flags & 2) ? noise : nullptr, s);
  double2 p = mom[s];
  if (flags & 1) {
    p.x -= gfac * f.g.x;
    p.y -= gfac * f.g.y;
  }
  if (chi != nullptr) {
    p.x -= eps * f.pf.x;
    p.y -= eps * f.pf.y;
  }
  if (flags & 2) {
    p.x -= eps * f.md.x;
    p.y -= eps * f.md.y;
  }
  mom[s] = p;
}

__global__ void __launch_bounds__(kBlock) k_force_field(Geo g, double ep, double em, const double2* __restrict__ A,
                                                        const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                        const double2* __restrict__ chi,
                                                        const double2* __restrict__ Mchi,
                                                        const double2* __restrict__ noise, double2* F, double gfac,
                                                        int flags) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= g.V) return;
  ForcePieces f = force_site(g, ep, em, A, Wt, Wx, chi, Mchi, (flags & 2) ? noise : nullptr, s);
  double2 o = F[s];
  if (flags & 1) {
    o.x += gfac * f.g.x;
    o.y += gfac * f.g.y;
  }
  o.x += f.pf.x + f.md.x;
  o.y += f.pf.y + f.md.y;
  F[s] = o;
}

void momentum_update(cudaStream_t s, const Geo& g, double ep, double em, const double2* A, const double2* Wt,
                     const double2* Wx, const double2* chi, const double2* Mchi, const double2* noise,
                     double2* mom, double eps, double gfac, int flags) {
  k_momentum_update<<<nblocks(g.V), kBlock, 0, s>>>(g, ep, em, A, Wt, Wx, chi, Mchi, noise, mom, eps, gfac, flags);
}
void force_field(cudaStream_t s, const Geo& g, double ep, double em, const double2* A, const double2* Wt,
                 const double2* Wx, const double2* chi, const double2* Mchi, const double2* noise, double2* F,
                 double gfac, int flags) {
  k_force_field<<<nblocks(g.V), kBlock, 0, s>>>(g, ep, em, A, Wt, Wx, chi, Mchi, noise, F, gfac, flags);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter = (site,
// stream, trajectory lo, trajectory hi), key = seed.  Each draw gives two
// 53-bit uniforms in (0,1) -> one Box-Muller pair.
// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(kBlock) k_philox_gauss(int n, unsigned long long seed, const TrajStats* ts,
                                                         unsigned stream_id, double2* out) {
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s >= n) return;
  unsigned long long tr = ts->traj;
  uint4 r = philox4x32(make_uint4((unsigned)s, stream_id, (unsigned)tr, (unsigned)(tr >> 32)),
                       make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
  double u1 = u53(r.x, r.y), u2 = u53(r.z, r.w);
  double rad = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  out[s] = make_double2(rad * cs, rad * sn);
}

__global__ void k_philox_uniform(unsigned long long seed, TrajStats* ts, unsigned stream_id) {
  unsigned long long tr = ts->traj;
  uint4 r = philox4x32(make_uint4(0xffffffffu, stream_id, (unsigned)tr, (unsigned)(tr >> 32)),
                       make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
  ts->u = u53(r.x, r.y);
}

void philox_gauss(cudaStream_t s, int n, unsigned long long seed, const TrajStats* ts, unsigned stream_id,
                  double2* out) {
  k_philox_gauss<<<nblocks(n), kBlock, 0, s>>>(n, seed, ts, stream_id, out);
}
void philox_uniform(cudaStream_t s, unsigned long long seed, TrajStats* ts, unsigned stream_id) {
  k_philox_uniform<<<1, 1, 0, s>>>(seed, ts, stream_id);
}

// Pure-gauge Metropolis (update_puregauge_hb, hmc.c:82-93): every link is
// independent (the compact action is a sum over single links), so one sweep is
// one data-parallel pass.  u holds the two uniforms of each link in the
// reference's order (proposal, then acceptance).  c = -Nf/g.  The proposal is
// computed without FMA contraction so it is bit-identical to the host's.
__global__ void __launch_bounds__(kBlock) k_puregauge(int n, double* A, const double* __restrict__ u, double c) {
  int k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= n) return;
  double a = A[k];
  double s1 = c * cos(a);
  double prop = __dsub_rn(__dmul_rn(2 * M_PI, u[2 * k]), M_PI);
  double s2 = c * cos(prop);
  if (u[2 * k + 1] < exp(-s2 + s1)) A[k] = prop;
}

void puregauge(cudaStream_t s, int nlinks, double* A, const double* u, double c) {
  k_puregauge<<<nblocks(nlinks), kBlock, 0, s>>>(nlinks, A, u, c);
}

// dH in the order of hmc.c:729-732, accept if exp(-dH) > u (hmc.c:738)
__global__ void k_finish(TrajStats* ts) {
  double dS = ts->Smom1 - ts->Smom0 + ts->Spf1 - ts->Spf0 + ts->Smd1 - ts->Smd0 + ts->Sg1 - ts->Sg0;
  ts->dH = dS;
  ts->accepted = exp(-dS) > ts->u ? 1 : 0;
  ts->traj += 1;
}

__global__ void __launch_bounds__(kBlock) k_accept_copy(int n, const TrajStats* ts, double2* A,
                                                        const double2* __restrict__ Anew) {
  if (!ts->accepted) return;
  int s = blockIdx.x * kBlock + threadIdx.x;
  if (s < n) A[s] = Anew[s];
}

void finish_trajectory(cudaStream_t s, TrajStats* ts) { k_finish<<<1, 1, 0, s>>>(ts); }
void accept_copy(cudaStream_t s, int n, const TrajStats* ts, double2* A, const double2* Anew) {
  k_accept_copy<<<nblocks(n), kBlock, 0, s>>>(n, ts, A, Anew);
}

}  // namespace tg
