// tg_aux.cu -- kernels beside the HMC path: measurements (hmc.c:794-842 and a
// stochastic chiral condensate) and the real, gauge-field-free, monomer-masked
// operator of the fermion-bag programs with its CG (vec_ops.c:96-174,
// 261-307).
#include <math.h>

#include "tg_device.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Measurements
// ---------------------------------------------------------------------------
// sum over sites of A_t + A_x (magnetisation numerator, hmc.c:831-833)
__global__ void __launch_bounds__(kBlock) k_sum_links(int n, const double2* __restrict__ A, double* dst, Red red) {
  double a = 0;
  TG_SITES(s, n) {
    double2 v = A[s];
    a += v.x + v.y;
  }
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = tot;
}

// Im <u, v> = sum (Re u Im v - Im u Re v)  (fermion_phase, hmc.c:805-808)
__global__ void __launch_bounds__(kBlock) k_imdot(int n, const double2* __restrict__ u, const double2* __restrict__ v,
                                                  double* dst, int acc, Red red) {
  double a = 0;
  TG_SITES(s, n) {
    double2 x = u[s], y = v[s];
    a += x.x * y.y - x.y * y.x;
  }
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0)
    *dst = acc ? *dst + tot : tot;
}

void sum_links(cudaStream_t s, const Geo& g, const double2* A, double* dst, const Red& red) {
  k_sum_links<<<g.grid, kBlock, 0, s>>>(g.V, A, dst, red);
}
void imdot(cudaStream_t s, const Geo& g, const double2* u, const double2* v, double* dst, int acc, const Red& red) {
  k_imdot<<<g.grid, kBlock, 0, s>>>(g.V, u, v, dst, acc, red);
}

// ---------------------------------------------------------------------------
// Masked real operator (vec_ops.c:96-174): mask[s] != 0 marks an occupied site,
// whose row is the identity and which is skipped as a neighbour.  fM: forward t
// hop +0.5 eta e^{mu}, backward t hop -0.5 eta e^{-mu}, x hops +-0.5, the sign of
// a hop that wraps multiplied by bc; fM^T negates the hops and swaps e^{+-mu}.
// ---------------------------------------------------------------------------
template <int TR>
__device__ __forceinline__ double fm_site(const Geo& g, double m, double ep, double em, int bc_t, int bc_x,
                                          const int* __restrict__ mask, const double* __restrict__ in, int s) {
  if (mask[s]) return in[s];
  int t, x;
  site_tx(g, s, t, x);
  Nbr n = neighbours(g, s, t, x);
  const double et = (x & 1) ? -0.5 : 0.5;
  const double sg = TR ? -1.0 : 1.0;
  const double fu = TR ? em : ep, fd = TR ? ep : em;
  double v = m * in[s];
  if (!mask[n.tp]) v += sg * et * fu * ((t == g.nt - 1) ? (double)bc_t : 1.0) * in[n.tp];
  if (!mask[n.tm]) v += sg * et * fd * ((t == 0) ? -(double)bc_t : -1.0) * in[n.tm];
  if (!mask[n.xp]) v += sg * 0.5 * ((x == g.nx - 1) ? (double)bc_x : 1.0) * in[n.xp];
  if (!mask[n.xm]) v += sg * 0.5 * ((x == 0) ? -(double)bc_x : -1.0) * in[n.xm];
  return v;
}

template <int TR>
__global__ void __launch_bounds__(kBlock) k_fm(Geo g, double m, double ep, double em, int bc_t, int bc_x,
                                               const int* __restrict__ mask, const double* __restrict__ in,
                                               double* __restrict__ out) {
  TG_SITES(s, g.V) out[s] = fm_site<TR>(g, m, ep, em, bc_t, bc_x, mask, in, s);
}

void fm_apply(cudaStream_t s, const Geo& g, double m, double mu, int bc_t, int bc_x, const int* mask,
              const double* in, double* out, int transpose) {
  const double ep = exp(mu), em = exp(-mu);
  if (transpose) k_fm<1><<<nblocks(g.V), kBlock, 0, s>>>(g, m, ep, em, bc_t, bc_x, mask, in, out);
  else k_fm<0><<<nblocks(g.V), kBlock, 0, s>>>(g, m, ep, em, bc_t, bc_x, mask, in, out);
}

// CG on fM^T fM (cg_MdM, vec_ops.c:261-307), state in a CgState as the complex solver.
__global__ void __launch_bounds__(kBlock) k_rcg_init(Geo g, const double* __restrict__ b, double* x, double* r,
                                                     double* p, double rel_tol, double abs_tol2, int maxiter,
                                                     CgState* st, Red red) {
  double v = 0;
  TG_SITES(s, g.V) {
    double bb = b[s];
    x[s] = 0;
    r[s] = bb;
    p[s] = bb;
    v += bb * bb;
  }
  double tot;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) {
    double stop = abs_tol2;
    if (rel_tol > 0 && rel_tol * rel_tol * tot > stop) stop = rel_tol * rel_tol * tot;
    st->rr = tot;
    st->rr0 = tot;
    st->stop = stop;
    st->iter = 0;
    st->maxiter = maxiter;
    st->status = TG_OK;
    st->log_index = -1;
    st->done = (!(tot >= stop) || tot == 0.0) ? 1 : 0;
    if (isnan(tot)) st->status = TG_E_NAN;
  }
}

// Ap = fM^T (fM p) needs fM p at the neighbours: tmp = fM p first (k_fm<0>), then this.
__global__ void __launch_bounds__(kBlock) k_rcg_ap(Geo g, double m, double ep, double em, int bc_t, int bc_x,
                                                   const int* __restrict__ mask, const double* __restrict__ tmp,
                                                   const double* __restrict__ p, double* __restrict__ Ap, CgState* st,
                                                   Red red) {
  if (st->done) return;
  double v = 0;
  TG_SITES(s, g.V) {
    double a = fm_site<1>(g, m, ep, em, bc_t, bc_x, mask, tmp, s);
    Ap[s] = a;
    v += p[s] * a;  // pMp = <p, fM^T fM p> (vec_ops.c:284)
  }
  double tot;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) st->alpha = st->rr / tot;
}

__global__ void __launch_bounds__(kBlock) k_rcg_fm_p(Geo g, double m, double ep, double em, int bc_t, int bc_x,
                                                     const int* __restrict__ mask, const double* __restrict__ p,
                                                     double* __restrict__ tmp, const CgState* st) {
  if (st->done) return;
  TG_SITES(s, g.V) tmp[s] = fm_site<0>(g, m, ep, em, bc_t, bc_x, mask, p, s);
}

__global__ void __launch_bounds__(kBlock) k_rcg_update(Geo g, const double* __restrict__ p,
                                                       const double* __restrict__ Ap, double* x, double* r,
                                                       CgState* st, Red red) {
  if (st->done) return;
  const double a = st->alpha;
  double v = 0;
  TG_SITES(s, g.V) {
    x[s] += a * p[s];
    double rv = r[s] - a * Ap[s];
    r[s] = rv;
    v += rv * rv;
  }
  double rn;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &rn) && threadIdx.x == 0) {
    st->iter += 1;
    st->beta = rn / st->rr;
    st->rr = rn;
    int status = -1;
    if (isnan(rn)) status = TG_E_NAN;
    else if (rn < st->stop) status = TG_OK;
    else if (rn / st->rr0 > 1e10) status = TG_E_DIVERGED;  // vec_ops.c:292-296
    else if (st->iter >= st->maxiter) status = TG_E_NOCONV;
    if (status >= 0) {
      st->status = status;
      st->done = 1;
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_rcg_p(int n, const double* __restrict__ r, double* p, const CgState* st) {
  if (st->done) return;
  const double b = st->beta;
  TG_SITES(s, n) p[s] = r[s] + b * p[s];
}

void rcg_init(cudaStream_t s, const Geo& g, const double* b, double* x, double* r, double* p, double rel_tol,
              double abs_tol2, int maxiter, CgState* st, const Red& red) {
  k_rcg_init<<<g.grid, kBlock, 0, s>>>(g, b, x, r, p, rel_tol, abs_tol2, maxiter, st, red);
}

void rcg_iter(cudaStream_t s, const Geo& g, double m, double mu, int bc_t, int bc_x, const int* mask, double* x,
              double* r, double* p, double* tmp, double* Ap, CgState* st, const Red& red) {
  const double ep = exp(mu), em = exp(-mu);
  k_rcg_fm_p<<<nblocks(g.V), kBlock, 0, s>>>(g, m, ep, em, bc_t, bc_x, mask, p, tmp, st);
  k_rcg_ap<<<g.grid, kBlock, 0, s>>>(g, m, ep, em, bc_t, bc_x, mask, tmp, p, Ap, st, red);
  k_rcg_update<<<g.grid, kBlock, 0, s>>>(g, p, Ap, x, r, st, red);
  k_rcg_p<<<nblocks(g.V), kBlock, 0, s>>>(g.V, r, p, st);
}

}  // namespace tg
