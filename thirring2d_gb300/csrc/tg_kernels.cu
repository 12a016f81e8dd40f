// tg_kernels.cu -- sm_103a kernels of the Thirring2D HMC hot path.
//
// Stencil kernels (operator applies and the CG kernels built on them) use the
// warp column march of stencil_all(): a warp walks a contiguous range of rows
// of 32 consecutive x, reusing psi(t-1), psi(t), Wt(t-1) from registers and
// taking x neighbours from warp shuffles, with the CG vector updates and norms
// fused into the per-site epilogue.  Lattices whose nx is not a multiple of 32 (or
// nt of kMarchT) use one site per thread.  Streaming kernels are one site per
// thread over the full grid.  Reductions are deterministic (fixed shuffle
// tree per block, partials summed in index order by the last block), so
// results do not depend on block scheduling.
#include <math.h>
#include <string.h>

#include <mutex>
#include <unordered_map>

#include "tg_stencil.cuh"

namespace tg {

// Minimum resident blocks per SM of the stencil kernels: FP32 ones are
// latency-bound and get more warps; FP64 ones are pipe-bound.
#define TG_FP32_BLOCKS_PER_SM 3
template <typename R> constexpr int kFp32BlocksPerSM = sizeof(R) == 4 ? TG_FP32_BLOCKS_PER_SM : kStencilBlocksPerSM;

__global__ void __launch_bounds__(kBlock) k_link_phase(Geo g, int bc_t, int bc_x, const double2* __restrict__ A,
                                                       LinkOut o) {
  TG_SITES(s, g.V) write_links(g, bc_t, bc_x, s, A[s], o);
}

// gauge_step (hmc.c:97-101) applied nadd times: A += c*p with c = 2*eps,
// product then sum (two roundings) as the reference's host code computes it.
__global__ void __launch_bounds__(kBlock) k_gauge_step(Geo g, int bc_t, int bc_x, double2* A,
                                                       const double2* __restrict__ mom, double c, int nadd,
                                                       LinkOut o) {
  TG_SITES(s, g.V) {
    double2 a = A[s];
    double2 p = mom[s];
    for (int k = 0; k < nadd; k++) {
      a.x = __dadd_rn(a.x, __dmul_rn(c, p.x));
      a.y = __dadd_rn(a.y, __dmul_rn(c, p.y));
    }
    A[s] = a;
    write_links(g, bc_t, bc_x, s, a, o);
  }
}

void link_phase(cudaStream_t s, const Geo& g, int bc_t, int bc_x, const double2* A, const LinkOut& o) {
  k_link_phase<<<stream_grid(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, A, o);
}
void gauge_step(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double2* A, const double2* mom, double c,
                int nadd, const LinkOut& o) {
  k_gauge_step<<<stream_grid(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, A, mom, c, nadd, o);
}

// Grid = resident blocks of this kernel on the GPU (one wave), at most `work`.
template <class K> int occ_grid(K kernel, int work) {
  static int sms = 0;
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  }
  auto it = cache.find((const void*)kernel);
  int per_sm;
  if (it == cache.end()) {
    per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm <= 0)
      per_sm = 1;
    cache.emplace((const void*)kernel, per_sm);
  } else {
    per_sm = it->second;
  }
  int grid = per_sm * sms;
  return grid < work ? grid : (work > 0 ? work : 1);
}

// The same with dynamic shared memory (staged kernels); the kernel's dynamic
// shared memory limit is raised to smem on first use.
template <class K> int occ_grid_smem(K kernel, int work, int smem) {
  static int sms = 0;
  static std::mutex mu;
  static std::unordered_map<const void*, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  }
  auto it = cache.find((const void*)kernel);
  int per_sm;
  if (it == cache.end()) {
    per_sm = 0;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess || per_sm <= 0)
      per_sm = 1;
    cache.emplace((const void*)kernel, per_sm);
  } else {
    per_sm = it->second;
  }
  int grid = per_sm * sms;
  return grid < work ? grid : (work > 0 ? work : 1);
}

// FP32 stencil kernels stage their rows through shared memory (TMA) on
// marching lattices when TG_STAGED=1 (read at every launch or capture).  Off
// by default: at 1024^2 and 2048^2 the staged apply measured 10.8 / 29.5 us
// against 8.8 / 27.3 us for register-fed loads (chunks per warp are too few
// for the copy pipeline to reach steady state).
bool staged_enabled(const Geo& g) {
  const char* e = getenv("TG_STAGED");
  return g.march && e && e[0] == '1';
}

template <typename R, int DAG, bool MU0, bool STAGED = false>
__global__ void __launch_bounds__(kBlock, kFp32BlocksPerSM<R>) k_dslash(Geo g, OpK<R> k, const C2<R>* __restrict__ in,
                                                   C2<R>* __restrict__ out, const C2<R>* __restrict__ Wt,
                                                   const C2<R>* __restrict__ Wx) {
  auto epi = [&](int s, C2<R> o, C2<R>) { out[s] = o; };
  if constexpr (STAGED) stencil_staged<R, DAG, MU0, false>(g, k, SrcOne<R>{in}, Wt, Wx, epi);
  else stencil_all<R, DAG, MU0>(g, k, in, Wt, Wx, epi);
}

// launch helper: picks the MU0 instance from the operator constants
#define TG_OP_DISPATCH(kk, LAUNCH)  \
  do {                              \
    if ((kk).mu0) {                 \
      constexpr bool MU0 = true;    \
      LAUNCH;                       \
    } else {                        \
      constexpr bool MU0 = false;   \
      LAUNCH;                       \
    }                               \
  } while (0)

void dslash64(cudaStream_t s, const Geo& g, const OpK<double>& k, int dag, const double2* in, double2* out,
              const double2* Wt, const double2* Wx) {
  const int w = stencil_work(g);
  if (dag)
    TG_OP_DISPATCH(k, (k_dslash<double, 1, MU0><<<occ_grid(k_dslash<double, 1, MU0>, w), kBlock, 0, s>>>(
                          g, k, in, out, Wt, Wx)));
  else
    TG_OP_DISPATCH(k, (k_dslash<double, 0, MU0><<<occ_grid(k_dslash<double, 0, MU0>, w), kBlock, 0, s>>>(
                          g, k, in, out, Wt, Wx)));
}
void dslash32(cudaStream_t s, const Geo& g, const OpK<float>& k, int dag, const float2* in, float2* out,
              const float2* Wt, const float2* Wx) {
  const int w = stencil_work(g);
  if (staged_enabled(g)) {
    constexpr int sm = staged_smem_bytes<float, 1>();
    if (dag)
      TG_OP_DISPATCH(k, (k_dslash<float, 1, MU0, true><<<occ_grid_smem(k_dslash<float, 1, MU0, true>, w, sm), kBlock,
                                                         sm, s>>>(g, k, in, out, Wt, Wx)));
    else
      TG_OP_DISPATCH(k, (k_dslash<float, 0, MU0, true><<<occ_grid_smem(k_dslash<float, 0, MU0, true>, w, sm), kBlock,
                                                         sm, s>>>(g, k, in, out, Wt, Wx)));
    return;
  }
  if (dag)
    TG_OP_DISPATCH(k, (k_dslash<float, 1, MU0><<<occ_grid(k_dslash<float, 1, MU0>, w), kBlock, 0, s>>>(
                          g, k, in, out, Wt, Wx)));
  else
    TG_OP_DISPATCH(k, (k_dslash<float, 0, MU0><<<occ_grid(k_dslash<float, 0, MU0>, w), kBlock, 0, s>>>(
                          g, k, in, out, Wt, Wx)));
}

// ---------------------------------------------------------------------------
// CG on M^dagger M (fmdm_invert_cg, hmc.c:341-404), one iteration =
//   K1: p' = r + beta p (formed on the fly for every operand the stencil
//       reads, stored at the own site), Mp = M p', pAp = |Mp|^2, alpha = rr/pAp
//   K2: x += alpha p', r -= alpha M^dag Mp, rr' = |r|^2, beta = rr'/rr, tests
// so the p update costs no pass of its own.  p lives in two buffers that
// alternate between consecutive iterations (p' cannot overwrite p while
// neighbouring sites still read it); the graph body holds two iterations.
// pAp = <p, M^dag M p> is taken as |Mp|^2 (same value, always >= 0).  The
// scalar recurrences run in the last block of K1/K2, so the host never waits.
// The FP32 instances (mixed precision) accumulate per-block sums in FP32 and
// combine the blocks in FP64.
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
  double v = 0;
  TG_SITES(s, g.V) {
    double2 bb = b[s];
    x[s] = make_double2(0.0, 0.0);
    C2<R> rb = mk<R>((R)bb.x, (R)bb.y);
    r[s] = rb;
    p[s] = rb;
    if (xs != nullptr) xs[s] = mk<R>(0, 0);
    v += bb.x * bb.x + bb.y * bb.y;
  }
  double tot;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) {
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

template <typename R, bool MU0, bool UNIT = false, bool STAGED = false>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? kFp32BlocksPerSM<R> : 2) k_cg1(Geo g, OpK<R> k, const C2<R>* __restrict__ r,
                                                const C2<R>* __restrict__ p_old, C2<R>* __restrict__ p_new,
                                                C2<R>* __restrict__ Mp, const C2<R>* __restrict__ Wt,
                                                const C2<R>* __restrict__ Wx, CgState* st, Red red) {
  if (st->done) return;
  const R b = (R)st->beta;
  R v = 0;
  auto ld = [&](int i) {
    const C2<R> rv = r[i], pv = p_old[i];
    return mk<R>(fma(b, pv.x, rv.x), fma(b, pv.y, rv.y));
  };
  auto epi = [&](int s, C2<R> o, C2<R> pc) {
    p_new[s] = pc;
    Mp[s] = o;
    v = fma(o.x, o.x, v);
    v = fma(o.y, o.y, v);
  };
  if constexpr (STAGED) stencil_staged<R, 0, MU0, UNIT>(g, k, SrcAxpy<R>{r, p_old, b}, Wt, Wx, epi);
  else stencil_ld<R, 0, MU0, UNIT>(g, k, ld, Wt, Wx, epi);
  double tot;
  if (grid_sum<kBlock, R>(v, red.partials, red.counter, &tot) && threadIdx.x == 0) {
    st->alpha = st->rr / tot;
    st->need_ru = 0;   // the previous iteration's reliable-update kernels have all run
    st->restart = 0;
  }
}

// FP64: convergence tested on the recursive residual, as hmc.c:381.
// UNIT: the pair runs CG on N^dag N with N = M / m (links W / m).  Its residual
// b - N^dag N (m^2 x) is b's residual for x, so r, p, beta and the stopping test
// are M's, and alpha_N = m^2 alpha_M: x advances by (alpha_N / m^2) p.
template <bool MU0, bool UNIT = false>
__global__ void __launch_bounds__(kBlock, 2) k_cg2_64(Geo g, OpK<double> k, const double2* __restrict__ Mp,
                                                   const double2* __restrict__ p, double2* __restrict__ x,
                                                   double2* __restrict__ r, const double2* __restrict__ Wt,
                                                   const double2* __restrict__ Wx, CgState* st, CgLog* log,
                                                   Red red, Cond c, double inv_m2 = 1.0) {
  if (st->done) return;
  const double a = st->alpha;
  const double ax = UNIT ? a * inv_m2 : a;
  double v = 0;
  auto epi = [&](int s, double2 ap, double2) {
    double2 xv = x[s], pv = p[s], rv = r[s];
    xv.x += ax * pv.x;
    xv.y += ax * pv.y;
    rv.x -= a * ap.x;
    rv.y -= a * ap.y;
    x[s] = xv;
    r[s] = rv;
    v = fma(rv.x, rv.x, v);
    v = fma(rv.y, rv.y, v);
  };
  stencil_all<double, 1, MU0, UNIT>(g, k, Mp, Wt, Wx, epi);
  double rn;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &rn) && threadIdx.x == 0) {
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

void cg64_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufs64& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int log_index, Cond c) {
  k_cg_init<double><<<occ_grid(k_cg_init<double>, nblocks(g.V)), kBlock, 0, s>>>(
      g, b, x, w.r, w.p[0], nullptr, rel_tol, abs_tol2, maxiter, 0, log_index, st, log, red, c);
}

void cg64_iter(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
               double2* x, const CgBufs64& w, int half, CgState* st, CgLog* log, const Red& red, Cond c) {
  const int wk = stencil_work(g);
  const double2* p_old = w.p[half];
  double2* p_new = w.p[half ^ 1];
  if (L.Wt1 != nullptr) {
    TG_OP_DISPATCH(km, (k_cg1<double, MU0, true><<<occ_grid(k_cg1<double, MU0, true>, wk), kBlock, 0, s>>>(
                            g, km, w.r, p_old, p_new, w.Mp, L.Wt1, L.Wx1, st, red)));
    TG_OP_DISPATCH(kd, (k_cg2_64<MU0, true><<<occ_grid(k_cg2_64<MU0, true>, wk), kBlock, 0, s>>>(
                            g, kd, w.Mp, p_new, x, w.r, L.Wt1, L.Wx1, st, log, red, c, L.inv_m2)));
    return;
  }
  TG_OP_DISPATCH(km, (k_cg1<double, MU0><<<occ_grid(k_cg1<double, MU0>, wk), kBlock, 0, s>>>(
                          g, km, w.r, p_old, p_new, w.Mp, L.Wt, L.Wx, st, red)));
  TG_OP_DISPATCH(kd, (k_cg2_64<MU0><<<occ_grid(k_cg2_64<MU0>, wk), kBlock, 0, s>>>(g, kd, w.Mp, p_new, x, w.r, L.Wt,
                                                                                 L.Wx, st, log, red, c)));
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 vectors and links, FP64 scalar recurrences.  x
// accumulates in FP64 at each reliable update, which recomputes
// r = b - M^dag M x in FP64 and restarts the FP32 residual from it.  Updates
// happen every ru_interval iterations, once |r|^2 has fallen by kRuDrop since
// the last one, when the FP32 residual reaches the target, and at the cap.
// ---------------------------------------------------------------------------
template <bool MU0, bool STAGED = false>
__global__ void __launch_bounds__(kBlock, kFp32BlocksPerSM<float>) k_cgmx2(Geo g, OpK<float> k, const float2* __restrict__ Mp,
                                                  const float2* __restrict__ p, float2* __restrict__ xs,
                                                  float2* __restrict__ r, const float2* __restrict__ Wt,
                                                  const float2* __restrict__ Wx, CgState* st, Red red, Cond c) {
  if (st->done) return;
  const float a = (float)st->alpha;
  float v = 0;
  auto epi = [&](int s, float2 ap, float2) {
    float2 xv = xs[s], pv = p[s], rv = r[s];
    xv.x = fmaf(a, pv.x, xv.x);
    xv.y = fmaf(a, pv.y, xv.y);
    rv.x = fmaf(-a, ap.x, rv.x);
    rv.y = fmaf(-a, ap.y, rv.y);
    xs[s] = xv;
    r[s] = rv;
    v = fmaf(rv.x, rv.x, v);
    v = fmaf(rv.y, rv.y, v);
  };
  if constexpr (STAGED) stencil_staged<float, 1, MU0, false>(g, k, SrcOne<float>{Mp}, Wt, Wx, epi);
  else stencil_all<float, 1, MU0>(g, k, Mp, Wt, Wx, epi);
  double rn;
  if (grid_sum<kBlock, float>(v, red.partials, red.counter, &rn) && threadIdx.x == 0) {
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
  TG_SITES(s, n) {
    float2 d = xs[s];
    double2 v = x[s];
    v.x += (double)d.x;
    v.y += (double)d.y;
    x[s] = v;
    xs[s] = make_float2(0.f, 0.f);
  }
}

// reliable update 2: tmp = M x (FP64)
template <bool MU0>
__global__ void __launch_bounds__(kBlock, kStencilBlocksPerSM) k_ru2(Geo g, OpK<double> k, const double2* __restrict__ x,
                                                double2* __restrict__ tmp, const double2* __restrict__ Wt,
                                                const double2* __restrict__ Wx, const CgState* st) {
  if (!st->need_ru || st->done) return;
  auto epi = [&](int s, double2 o, double2) { tmp[s] = o; };
  stencil_all<double, 0, MU0>(g, k, x, Wt, Wx, epi);
}

// reliable update 3: r = b - M^dag tmp (FP64), rs = (float) r, decide
template <bool MU0>
__global__ void __launch_bounds__(kBlock, kStencilBlocksPerSM) k_ru3(Geo g, OpK<double> k, const double2* __restrict__ b,
                                                const double2* __restrict__ tmp, float2* __restrict__ rs,
                                                const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                CgState* st, CgLog* log, Red red, Cond c) {
  if (!st->need_ru || st->done) return;
  double v = 0;
  auto epi = [&](int s, double2 ap, double2) {
    double2 bb = b[s];
    double2 rv = make_double2(bb.x - ap.x, bb.y - ap.y);
    rs[s] = make_float2((float)rv.x, (float)rv.y);
    v = fma(rv.x, rv.x, v);
    v = fma(rv.y, rv.y, v);
  };
  stencil_all<double, 1, MU0>(g, k, tmp, Wt, Wx, epi);
  double rt;
  if (grid_sum<kBlock, double>(v, red.partials, red.counter, &rt) && threadIdx.x == 0) {
    st->restart = rt > kRuRestart * st->rr;  // recursive residual was far too optimistic:
    if (st->restart) st->beta = 0;            // the next p starts again from r
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

void cgmx_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufsMixed& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int ru_interval,
               int log_index, Cond c) {
  k_cg_init<float><<<occ_grid(k_cg_init<float>, nblocks(g.V)), kBlock, 0, s>>>(
      g, b, x, w.rs, w.ps[0], w.xs, rel_tol, abs_tol2, maxiter, ru_interval, log_index, st, log, red, c);
}

void cgmx_iter(cudaStream_t s, const Geo& g, const OpK<float>& km, const OpK<float>& kd, const Links& L,
               const CgBufsMixed& w, int half, CgState* st, const Red& red, Cond c) {
  const int wk = stencil_work(g);
  const float2* p_old = w.ps[half];
  float2* p_new = w.ps[half ^ 1];
  if (staged_enabled(g)) {
    constexpr int sm1 = staged_smem_bytes<float, 2>(), sm2 = staged_smem_bytes<float, 1>();
    TG_OP_DISPATCH(km, (k_cg1<float, MU0, false, true><<<occ_grid_smem(k_cg1<float, MU0, false, true>, wk, sm1),
                                                         kBlock, sm1, s>>>(g, km, w.rs, p_old, p_new, w.Mps, L.Wt32,
                                                                           L.Wx32, st, red)));
    TG_OP_DISPATCH(kd, (k_cgmx2<MU0, true><<<occ_grid_smem(k_cgmx2<MU0, true>, wk, sm2), kBlock, sm2, s>>>(
                            g, kd, w.Mps, p_new, w.xs, w.rs, L.Wt32, L.Wx32, st, red, c)));
    return;
  }
  TG_OP_DISPATCH(km, (k_cg1<float, MU0><<<occ_grid(k_cg1<float, MU0>, wk), kBlock, 0, s>>>(
                          g, km, w.rs, p_old, p_new, w.Mps, L.Wt32, L.Wx32, st, red)));
  TG_OP_DISPATCH(kd, (k_cgmx2<MU0><<<occ_grid(k_cgmx2<MU0>, wk), kBlock, 0, s>>>(g, kd, w.Mps, p_new, w.xs, w.rs,
                                                                               L.Wt32, L.Wx32, st, red, c)));
}

void cgmx_reliable(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
                   const double2* b, double2* x, const CgBufsMixed& w, CgState* st, CgLog* log, const Red& red,
                   Cond c) {
  const int wk = stencil_work(g);
  k_ru1<<<stream_grid(g.V), kBlock, 0, s>>>(g.V, x, w.xs, st);
  TG_OP_DISPATCH(km, (k_ru2<MU0><<<occ_grid(k_ru2<MU0>, wk), kBlock, 0, s>>>(g, km, x, w.tmp64, L.Wt, L.Wx, st)));
  TG_OP_DISPATCH(kd, (k_ru3<MU0><<<occ_grid(k_ru3<MU0>, wk), kBlock, 0, s>>>(g, kd, b, w.tmp64, w.rs, L.Wt, L.Wx, st,
                                                                           log, red, c)));
}

// ---------------------------------------------------------------------------
// Reductions for the Hamiltonian (hmc.c:73-79, 428, 451-463, 467-479, 493, 723)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_norm2(int n, const double2* __restrict__ v, double* dst, int acc,
                                                  Red red) {
  double a = 0;
  TG_SITES(s, n) {
    double2 u = v[s];
    a += u.x * u.x + u.y * u.y;
  }
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0)
    *dst = acc ? *dst + tot : tot;
}

__global__ void __launch_bounds__(kBlock) k_redot(int n, const double2* __restrict__ u, const double2* __restrict__ v,
                                                  double* dst, int acc, Red red) {
  double a = 0;
  TG_SITES(s, n) {
    double2 x = u[s], y = v[s];
    a += x.x * y.x + x.y * y.y;
  }
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0)
    *dst = acc ? *dst + tot : tot;
}

__global__ void __launch_bounds__(kBlock) k_gauge_action(int n, const double2* __restrict__ A, double fac,
                                                         double* dst, Red red) {
  double a = 0;
  TG_SITES(s, n) {
    double2 v = A[s];
    a += (1. - cos(v.x)) + (1. - cos(v.y));
  }
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = fac * tot;
}

template <bool MU0>
__global__ void __launch_bounds__(kBlock, kStencilBlocksPerSM) k_md_action(Geo g, OpK<double> k, const double2* __restrict__ nz,
                                                      const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                      double* dst, Red red) {
  double a = 0;
  auto epi = [&](int, double2 o, double2 v) { a += v.x * o.x + v.y * o.y; };
  stencil_all<double, 1, MU0>(g, k, nz, Wt, Wx, epi);
  double tot;
  if (grid_sum<kBlock, double>(a, red.partials, red.counter, &tot) && threadIdx.x == 0) *dst = tot;
}

void norm2(cudaStream_t s, const Geo& g, const double2* v, double* dst, int accumulate, const Red& red) {
  k_norm2<<<occ_grid(k_norm2, nblocks(g.V)), kBlock, 0, s>>>(g.V, v, dst, accumulate, red);
}
void redot(cudaStream_t s, const Geo& g, const double2* u, const double2* v, double* dst, int accumulate,
           const Red& red) {
  k_redot<<<occ_grid(k_redot, nblocks(g.V)), kBlock, 0, s>>>(g.V, u, v, dst, accumulate, red);
}
void gauge_action(cudaStream_t s, const Geo& g, const double2* A, double fac, double* dst, const Red& red) {
  k_gauge_action<<<occ_grid(k_gauge_action, nblocks(g.V)), kBlock, 0, s>>>(g.V, A, fac, dst, red);
}
void md_action(cudaStream_t s, const Geo& g, const OpK<double>& kd, const double2* nz, const double2* Wt,
               const double2* Wx, double* dst, const Red& red) {
  TG_OP_DISPATCH(kd, (k_md_action<MU0><<<occ_grid(k_md_action<MU0>, stencil_work(g)), kBlock, 0, s>>>(
                          g, kd, nz, Wt, Wx, dst, red)));
}

// ---------------------------------------------------------------------------
// Force (momentum_step, hmc.c:504-661), per link:
//   gauge   (Nf/g) sin A                                           (507-510)
//   pf      2 Im W (e^{mu} conj(Mchi(s)) chi(s+mu) - e^{-mu} conj(chi(s)) Mchi(s+mu))   (517-576)
//   noise   -(e^{mu} - e^{-mu}) Im W conj(n(s)) n(s+t), t links only  (608-661)
// with e^{+-mu} on t links only.  The three parts are subtracted from p in
// the reference's order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_momentum_update(Geo g, int bc_t, int bc_x, double ep, double em,
                                                            const double2* __restrict__ A,
                                                            const double2* __restrict__ Wt,
                                                            const double2* __restrict__ Wx,
                                                            const double2* __restrict__ chi,
                                                            const double2* __restrict__ Mchi,
                                                            const double2* __restrict__ noise, double2* mom,
                                                            double eps, double gfac, int flags) {
  TG_SITES(s, g.V) {
    ForcePieces f = force_site(g, bc_t, bc_x, ep, em, A, Wt, Wx, chi, Mchi, (flags & 2) ? noise : nullptr, s);
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
}

__global__ void __launch_bounds__(kBlock) k_force_field(Geo g, int bc_t, int bc_x, double ep, double em,
                                                        const double2* __restrict__ A,
                                                        const double2* __restrict__ Wt, const double2* __restrict__ Wx,
                                                        const double2* __restrict__ chi,
                                                        const double2* __restrict__ Mchi,
                                                        const double2* __restrict__ noise, double2* F, double gfac,
                                                        int flags) {
  TG_SITES(s, g.V) {
    ForcePieces f = force_site(g, bc_t, bc_x, ep, em, A, Wt, Wx, chi, Mchi, (flags & 2) ? noise : nullptr, s);
    double2 o = F[s];
    if (flags & 1) {
      o.x += gfac * f.g.x;
      o.y += gfac * f.g.y;
    }
    o.x += f.pf.x + f.md.x;
    o.y += f.pf.y + f.md.y;
    F[s] = o;
  }
}

void momentum_update(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double ep, double em, const double2* A,
                     const double2* Wt, const double2* Wx, const double2* chi, const double2* Mchi,
                     const double2* noise, double2* mom, double eps, double gfac, int flags) {
  k_momentum_update<<<stream_grid(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, ep, em, A, Wt, Wx, chi, Mchi, noise, mom, eps,
                                                        gfac, flags);
}
void force_field(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double ep, double em, const double2* A,
                 const double2* Wt, const double2* Wx, const double2* chi, const double2* Mchi, const double2* noise,
                 double2* F, double gfac, int flags) {
  k_force_field<<<stream_grid(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, ep, em, A, Wt, Wx, chi, Mchi, noise, F, gfac,
                                                    flags);
}

// ---------------------------------------------------------------------------
// Random fields (Philox, tg_device.cuh)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_philox_gauss(int n, unsigned long long seed, const TrajStats* ts,
                                                         unsigned stream_id, double2* out) {
  const unsigned long long tr = ts->traj;
  TG_SITES(s, n) out[s] = philox_gauss_pair(seed, tr, (unsigned)s, stream_id);
}

__global__ void k_philox_uniform(unsigned long long seed, TrajStats* ts, unsigned stream_id) {
  ts->u = philox_uniform1(seed, ts->traj, stream_id);
}

void philox_gauss(cudaStream_t s, const Geo& g, unsigned long long seed, const TrajStats* ts, unsigned stream_id,
                  double2* out) {
  k_philox_gauss<<<stream_grid(g.V), kBlock, 0, s>>>(g.V, seed, ts, stream_id, out);
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
  TG_SITES(k, n) {
    double a = A[k];
    double s1 = c * cos(a);
    double prop = __dsub_rn(__dmul_rn(2 * M_PI, u[2 * k]), M_PI);
    double s2 = c * cos(prop);
    if (u[2 * k + 1] < exp(-s2 + s1)) A[k] = prop;
  }
}

void puregauge(cudaStream_t s, const Geo& g, double* A, const double* u, double c) {
  k_puregauge<<<stream_grid(2 * g.V), kBlock, 0, s>>>(2 * g.V, A, u, c);
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
  TG_SITES(s, n) A[s] = Anew[s];
}

void finish_trajectory(cudaStream_t s, TrajStats* ts) { k_finish<<<1, 1, 0, s>>>(ts); }
void accept_copy(cudaStream_t s, const Geo& g, const TrajStats* ts, double2* A, const double2* Anew) {
  k_accept_copy<<<stream_grid(g.V), kBlock, 0, s>>>(g.V, ts, A, Anew);
}

}  // namespace tg

namespace tg {

// ---------------------------------------------------------------------------
// Launchers with an explicit grid, for callers that must not touch the
// occupancy cache above (it grows a host-side map): the allocation-free CG
// entry point (tg_noalloc.cu).  Same kernels, same arithmetic.
// ---------------------------------------------------------------------------
int resident_grid_nocache(const void* kernel, int work) {
  int dev = 0, sms = 1, per_sm = 1;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm <= 0)
    per_sm = 1;
  const int grid = per_sm * sms;
  return grid < work ? grid : (work > 0 ? work : 1);
}

void link_phase_fixed(cudaStream_t s, const Geo& g, int bc_t, int bc_x, const double2* A, double2* Wt, double2* Wx,
                      float2* Wt32, float2* Wx32) {
  k_link_phase<<<stream_grid(g.V), kBlock, 0, s>>>(g, bc_t, bc_x, A, LinkOut{Wt, Wx, Wt32, Wx32});
}

void cg64_init_fixed(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufs64& w, CgState* st,
                     const Red& red, double rel_tol, double abs_tol2, int maxiter) {
  const int grid = resident_grid_nocache((const void*)k_cg_init<double>, nblocks(g.V));
  k_cg_init<double><<<grid, kBlock, 0, s>>>(g, b, x, w.r, w.p[0], nullptr, rel_tol, abs_tol2, maxiter, 0, -1, st,
                                            nullptr, red, Cond{0, 0, 0});
}

void cg64_iter_fixed(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
                     double2* x, const CgBufs64& w, int half, CgState* st, const Red& red) {
  const int wk = stencil_work(g);
  const double2* p_old = w.p[half];
  double2* p_new = w.p[half ^ 1];
  TG_OP_DISPATCH(km, (k_cg1<double, MU0><<<resident_grid_nocache((const void*)k_cg1<double, MU0>, wk), kBlock, 0,
                                          s>>>(g, km, w.r, p_old, p_new, w.Mp, L.Wt, L.Wx, st, red)));
  TG_OP_DISPATCH(kd, (k_cg2_64<MU0><<<resident_grid_nocache((const void*)k_cg2_64<MU0>, wk), kBlock, 0, s>>>(
                          g, kd, w.Mp, p_new, x, w.r, L.Wt, L.Wx, st, nullptr, red, Cond{0, 0, 0})));
}

// Stage waits of the staged kernels of this file that ran out (0 in a healthy run).
unsigned stage_faults() {
  unsigned v = 0;
  if (cudaMemcpyFromSymbol(&v, g_stage_faults, sizeof v) != cudaSuccess) return 0xffffffffu;
  return v;
}

}  // namespace tg
