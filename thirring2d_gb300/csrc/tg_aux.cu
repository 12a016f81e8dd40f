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

namespace tg {

// ---------------------------------------------------------------------------
// Dense M and its determinant for tiny lattices (fermion_matrix and
// determinant, hmc.c:269-336).  Row-major: (M psi)_i = sum_j Md[i*V + j] psi_j,
// the same operator as the stencil (entries accumulate, so sides of 2, whose
// two neighbours coincide, are built correctly).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_dense_M(Geo g, OpK<double> k, const double2* __restrict__ Wt,
                                                   const double2* __restrict__ Wx, double2* __restrict__ Md) {
  const long long V = g.V;
  TG_SITES(i, g.V) {
    double2* row = Md + (long long)i * V;
    for (long long j = 0; j < V; j++) row[j] = make_double2(0, 0);
    int t, x;
    site_tx(g, i, t, x);
    Nbr n = neighbours(g, i, t, x);
    auto add = [&](int j, double2 v) {
      row[j].x += v.x;
      row[j].y += v.y;
    };
    add(i, make_double2(k.m, 0));
    double2 w = Wt[i];
    add(n.tp, make_double2(k.cf * w.x, k.cf * w.y));         // cf * Wt(s)
    w = Wt[n.tm];
    add(n.tm, make_double2(k.cb * w.x, -k.cb * w.y));        // cb * conj(Wt(s-t))
    w = Wx[i];
    add(n.xp, w);                                            // + Wx(s)
    w = Wx[n.xm];
    add(n.xm, make_double2(-w.x, w.y));                      // - conj(Wx(s-x))
  }
}

// LU with partial pivoting of one V x V complex matrix per block (in place).
// out[2*b] = log|det|, out[2*b+1] = arg(det) in (-pi, pi].
__global__ void __launch_bounds__(1024) k_lu_logdet(int V, double2* __restrict__ mats, double* __restrict__ out) {
  double2* a = mats + (long long)blockIdx.x * V * V;
  __shared__ double s_mag[1024];
  __shared__ int s_idx[1024];
  __shared__ int piv;
  double logabs = 0, ph = 0;  // valid in thread 0
  for (int k = 0; k < V; k++) {
    // pivot: largest |a_ik|, i >= k (ties to the smallest index: deterministic)
    double best = -1;
    int bi = k;
    for (int i = k + threadIdx.x; i < V; i += blockDim.x) {
      double2 v = a[(long long)i * V + k];
      double mag = v.x * v.x + v.y * v.y;
      if (mag > best) { best = mag; bi = i; }
    }
    s_mag[threadIdx.x] = best;
    s_idx[threadIdx.x] = bi;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < off) {
        double o = s_mag[threadIdx.x + off];
        int oi = s_idx[threadIdx.x + off];
        if (o > s_mag[threadIdx.x] || (o == s_mag[threadIdx.x] && oi < s_idx[threadIdx.x])) {
          s_mag[threadIdx.x] = o;
          s_idx[threadIdx.x] = oi;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) piv = s_idx[0];
    __syncthreads();
    const int p = piv;
    if (p != k) {
      for (int j = threadIdx.x; j < V; j += blockDim.x) {
        double2 u = a[(long long)k * V + j];
        a[(long long)k * V + j] = a[(long long)p * V + j];
        a[(long long)p * V + j] = u;
      }
      if (threadIdx.x == 0) ph += M_PI;  // a row swap flips the sign
    }
    __syncthreads();
    const double2 d = a[(long long)k * V + k];
    if (threadIdx.x == 0) {
      logabs += 0.5 * log(d.x * d.x + d.y * d.y);
      ph += atan2(d.y, d.x);
    }
    const double inv = 1.0 / (d.x * d.x + d.y * d.y);
    const double2 dinv = make_double2(d.x * inv, -d.y * inv);
    // eliminate below the pivot: a_ij -= (a_ik / a_kk) a_kj, i, j > k
    const int rows = V - k - 1;
    const long long work = (long long)rows * (V - k);
    for (long long w = threadIdx.x; w < work; w += blockDim.x) {
      const int i = k + 1 + (int)(w / (V - k));
      const int j = k + (int)(w % (V - k));
      double2 aik = a[(long long)i * V + k];
      double2 l = cmul<double>(aik, dinv);
      if (j == k) continue;  // column k is finished after the update below
      double2 akj = a[(long long)k * V + j];
      double2& aij = a[(long long)i * V + j];
      aij.x -= l.x * akj.x - l.y * akj.y;
      aij.y -= l.x * akj.y + l.y * akj.x;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ph = remainder(ph, 2 * M_PI);
    out[2 * blockIdx.x] = logabs;
    out[2 * blockIdx.x + 1] = ph;
  }
}

void dense_M(cudaStream_t s, const Geo& g, const OpK<double>& k, const double2* Wt, const double2* Wx, double2* Md) {
  k_dense_M<<<nblocks(g.V), kBlock, 0, s>>>(g, k, Wt, Wx, Md);
}
void lu_logdet(cudaStream_t s, int V, int nmat, double2* mats, double* out) {
  k_lu_logdet<<<nmat, 1024, 0, s>>>(V, mats, out);
}

}  // namespace tg

namespace tg {

// ---------------------------------------------------------------------------
// FP64 FMA throughput of this GPU: 8 independent dependent chains per thread,
// 4 blocks of 256 threads per SM.  The store is conditional on a value the
// chains never reach, so nothing is eliminated and nothing is written.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_dfma_peak(int iters, double seed, double* sink) {
  const double b = 0.9999999, c = 1e-9;
  double a0 = seed + threadIdx.x * 1e-12, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
  double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
      a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == -1.0) sink[0] = s;
}

// FMA count of one launch: grid * 256 threads * 8 chains * 4 * iters
void dfma_peak(cudaStream_t s, int grid, int iters, double* sink) {
  k_dfma_peak<<<grid, 256, 0, s>>>(iters, 1.0, sink);
}

}  // namespace tg

namespace tg {

// ---------------------------------------------------------------------------
// Propagator matrix of the fermion-bag programs: calc_Dinv with
// WITH_MASS_MONOMERS (fermion_matrix.c:189-351).  For every source site the
// column fM^-1 e_src comes from cg_propagator (vec_ops.c:311-321): CG on
// fM^T fM (vec_ops.c:261-307) with b = fM^T e_src.  One block per source, all
// of a launch's sources at once; every block keeps x, r, p, fM p, fM^T fM p in
// its own slice of `scratch`.  The entries on the sites of the other parity
// go to Dinv as the reference stores them (n = V/2, i = (nx*t + x)/2):
//   Dinv[i2*n + i1]       odd source i1, even site i2
//   Dinv[n*n + i2*n + i1] even source i1, odd site i2
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_allsum(double v) {
  __shared__ double sh[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // the previous call's readers are done with sh
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double t = 0;
  for (int i = 0; i < nw; i++) t += sh[i];  // same order in every thread
  return t;
}

__global__ void __launch_bounds__(kBlock) k_prop_cg(PropArgs a) {
  const Geo& g = a.g;
  const int V = g.V;
  const int src = a.src0 + blockIdx.x;
  double* x = a.scratch + (size_t)blockIdx.x * 5 * V;
  double* r = x + V;
  double* p = r + V;
  double* Mp = p + V;
  double* MMp = Mp + V;
  for (int s = threadIdx.x; s < V; s += blockDim.x) {
    Mp[s] = (s == src) ? 1.0 : 0.0;
    x[s] = 0.0;
  }
  __syncthreads();
  double v = 0;
  for (int s = threadIdx.x; s < V; s += blockDim.x) {  // r = p = fM^T e_src
    const double b = fm_site<1>(g, a.m, a.ep, a.em, a.bc_t, a.bc_x, a.mask, Mp, s);
    r[s] = b;
    p[s] = b;
    v = fma(b, b, v);
  }
  double rr_old = block_allsum(v);
  const double rr_init = rr_old;
  double stop = a.abs_tol2;
  if (a.rel_tol > 0 && a.rel_tol * a.rel_tol * rr_init > stop) stop = a.rel_tol * a.rel_tol * rr_init;
  int status = TG_OK, iters = 0;
  if (!(rr_old < stop)) {  // vec_ops.c:275-277
    status = TG_E_NOCONV;
    while (iters < a.maxiter) {
      __syncthreads();
      for (int s = threadIdx.x; s < V; s += blockDim.x)
        Mp[s] = fm_site<0>(g, a.m, a.ep, a.em, a.bc_t, a.bc_x, a.mask, p, s);
      __syncthreads();
      v = 0;
      for (int s = threadIdx.x; s < V; s += blockDim.x) {
        const double mm = fm_site<1>(g, a.m, a.ep, a.em, a.bc_t, a.bc_x, a.mask, Mp, s);
        MMp[s] = mm;
        v = fma(p[s], mm, v);
      }
      const double alpha = rr_old / block_allsum(v);  // rr / <p, fM^T fM p>
      v = 0;
      for (int s = threadIdx.x; s < V; s += blockDim.x) {
        x[s] = fma(alpha, p[s], x[s]);
        const double rv = fma(-alpha, MMp[s], r[s]);
        r[s] = rv;
        v = fma(rv, rv, v);
      }
      const double rr = block_allsum(v);
      iters++;
      if (isnan(rr)) {
        status = TG_E_NAN;
        break;
      }
      if (rr < stop) {
        status = TG_OK;
        break;
      }
      if (rr / rr_init > 1e10) {  // an (almost) exact zero mode: vec_ops.c:292-296 sets the solution to 1e50
        status = TG_E_DIVERGED;
        for (int s = threadIdx.x; s < V; s += blockDim.x) x[s] = 1e50;
        break;
      }
      const double beta = rr / rr_old;
      for (int s = threadIdx.x; s < V; s += blockDim.x) p[s] = fma(beta, p[s], r[s]);
      rr_old = rr;
    }
  }
  __syncthreads();
  int ts, xs;
  site_tx(g, src, ts, xs);
  const int par = (ts + xs) & 1;
  const int n = V / 2;
  double* out = a.Dinv + (par ? 0 : (size_t)n * n);
  const int i1 = src / 2;
  for (int s = threadIdx.x; s < V; s += blockDim.x) {
    int t, xx;
    site_tx(g, s, t, xx);
    if (((t + xx) & 1) != par) out[(size_t)(s / 2) * n + i1] = x[s];
  }
  if (threadIdx.x == 0) {
    atomicMax(a.max_iter, iters);
    atomicMax(a.worst, status);
  }
}

void prop_cg(cudaStream_t s, int nsrc, const PropArgs& a) { k_prop_cg<<<nsrc, kBlock, 0, s>>>(a); }

}  // namespace tg
