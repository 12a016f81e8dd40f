// tg_internal.cuh -- shared device/host definitions of the Thirring2D GB300 library.
//
// Layout in HBM (one lattice, V = nt*nx sites, site s = t*nx + x, t-major as
// in the reference hmc.c loops):
//   gauge field A        double2[V]   (.x = A_t, .y = A_x)   hmc.c A[t][x][dir]
//   momenta              double2[V]   (.x = p_t, .y = p_x)
//   fermion vectors      double2[V] / float2[V]  (re, im)    hmc.c v[t][x]
//   link coefficients    Wt[V], Wx[V] (complex, FP64 and FP32 copies)
//                        W_mu(s) = 0.5 * eta_mu(s) * bc_mu(s) * exp(i A_mu(s))
//                        i.e. every real factor of a hop in hmc.c:140-180
//                        except exp(+-mu) is folded in once per gauge update.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/thirring_gpu.h"

namespace tg {

constexpr int kBlock = 256;        // threads per block for site kernels
constexpr int kNf = 2;             // flavours in the gauge action, hmc.c:28

template <typename R> struct C2T;
template <> struct C2T<double> { using type = double2; };
template <> struct C2T<float> { using type = float2; };
template <typename R> using C2 = typename C2T<R>::type;

template <typename R> __host__ __device__ __forceinline__ C2<R> mk(R a, R b) { C2<R> v; v.x = a; v.y = b; return v; }

// acc += w * v
template <typename R> __device__ __forceinline__ void cmac(C2<R>& acc, C2<R> w, C2<R> v) {
  acc.x = fma(w.x, v.x, acc.x); acc.x = fma(-w.y, v.y, acc.x);
  acc.y = fma(w.x, v.y, acc.y); acc.y = fma(w.y, v.x, acc.y);
}
// acc -= w * v
template <typename R> __device__ __forceinline__ void cnmac(C2<R>& acc, C2<R> w, C2<R> v) {
  acc.x = fma(-w.x, v.x, acc.x); acc.x = fma(w.y, v.y, acc.x);
  acc.y = fma(-w.x, v.y, acc.y); acc.y = fma(-w.y, v.x, acc.y);
}
// acc += conj(w) * v
template <typename R> __device__ __forceinline__ void cjmac(C2<R>& acc, C2<R> w, C2<R> v) {
  acc.x = fma(w.x, v.x, acc.x); acc.x = fma(w.y, v.y, acc.x);
  acc.y = fma(w.x, v.y, acc.y); acc.y = fma(-w.y, v.x, acc.y);
}
// acc -= conj(w) * v
template <typename R> __device__ __forceinline__ void cmsc(C2<R>& acc, C2<R> w, C2<R> v) {
  acc.x = fma(-w.x, v.x, acc.x); acc.x = fma(-w.y, v.y, acc.x);
  acc.y = fma(-w.x, v.y, acc.y); acc.y = fma(w.y, v.x, acc.y);
}
// w * v
template <typename R> __device__ __forceinline__ C2<R> cmul(C2<R> w, C2<R> v) {
  return mk<R>(fma(w.x, v.x, -w.y * v.y), fma(w.x, v.y, w.y * v.x));
}
// conj(w) * v
template <typename R> __device__ __forceinline__ C2<R> cjmul(C2<R> w, C2<R> v) {
  return mk<R>(fma(w.x, v.x, w.y * v.y), fma(w.x, v.y, -w.y * v.x));
}

// Lattice geometry for kernels (by value).
struct Geo {
  int nt, nx, V;
  float inv_nx;   // for the division-free site -> (t, x) split
  int grid;       // blocks of a reducing site kernel: min(ceil(V/256), resident blocks of the GPU)
  int march;      // 1: stencil kernels use the warp column march (nx % 32 == 0, nt % kMarchT == 0)
  int mgrid;      // blocks of a column-march kernel
};

// Column march: a warp owns 32 consecutive x and walks its range of rows in t
// kMarchT rows at a time, keeping psi(t-1), psi(t) and Wt(t-1) in registers;
// the x neighbours come from warp shuffles (the operands across the warp's
// edges are fetched once per kMarchT rows by the first lanes).  Per site that
// leaves 3 coalesced loads (psi(t+1), Wt, Wx) instead of 9.
constexpr int kMarchT = 4;
// Minimum resident blocks per SM the stencil kernels are compiled for.
constexpr int kStencilBlocksPerSM = 1;  // no register cap: capping at 42 spilled heavily

__device__ __forceinline__ void site_tx(const Geo& g, int s, int& t, int& x) {
  // V < 2^24 keeps float(s) exact; the fix-up absorbs the rounding of s/nx.
  t = __float2int_rz(__int2float_rn(s) * g.inv_nx);
  x = s - t * g.nx;
  if (x < 0) { t -= 1; x += g.nx; } else if (x >= g.nx) { t += 1; x -= g.nx; }
}

struct Nbr { int tp, tm, xp, xm; };
__device__ __forceinline__ Nbr neighbours(const Geo& g, int s, int t, int x) {
  Nbr n;
  n.tp = (t == g.nt - 1) ? s + g.nx - g.V : s + g.nx;
  n.tm = (t == 0) ? s - g.nx + g.V : s - g.nx;
  n.xp = (x == g.nx - 1) ? s - (g.nx - 1) : s + 1;
  n.xm = (x == 0) ? s + (g.nx - 1) : s - 1;
  return n;
}

// Operator constants for M (dag = 0) or the true adjoint M^dagger (dag = 1):
//   out = m in + cf*Wt in(s+t) + cb*conj(Wt(s-t)) in(s-t) + sx*(Wx in(s+x) - conj(Wx(s-x)) in(s-x))
// M: cf = e^mu, cb = -e^-mu, sx = +1 (hmc.c:137-180); M^dag: cf = -e^-mu, cb = e^mu, sx = -1.
// sx is a template parameter of the kernels; mu0 = (mu == 0) selects the
// variant without the e^{+-mu} multiplies (18 instead of 22 FMA/MUL per site).
template <typename R> struct OpK {
  R m, cf, cb;
  int mu0;
};

// ---------------------------------------------------------------------------
// Block reduction (deterministic: fixed shuffle tree, then fixed smem order)
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int BS, typename T> __device__ __forceinline__ T block_sum(T v, T* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (w == 0) {
    r = (lane < BS / 32) ? sh[lane] : T(0);
    r = warp_sum(r);
  }
  __syncthreads();
  return r;  // valid in thread 0
}

// Grid-wide deterministic sum with the "last block finishes" pattern: every
// block stores its partial (summed in T: float for the FP32 solver, double
// otherwise), the block that arrives last adds the partials in FP64 in index
// order.  Returns true in exactly one block (all its threads), with the total
// in *total (thread 0 of that block).  `counter` must be 0 on entry and is 0
// again on exit.  Grids are capped near the resident-block count, so the
// serial part (one atomic per block, one pass over the partials) stays short.
template <int BS, typename T>
__device__ __forceinline__ bool grid_sum(T v, double* partials, unsigned* counter, double* total) {
  __shared__ T sh[BS / 32];
  __shared__ double shd[BS / 32];
  __shared__ bool is_last;
  T b = block_sum<BS, T>(v, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = (double)b;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double s = 0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += BS) s += __ldcg(partials + i);
  s = block_sum<BS, double>(s, shd);
  if (threadIdx.x == 0) {
    *total = s;
    *counter = 0u;
  }
  return true;
}

inline int nblocks(int n, int bs = kBlock) { return (n + bs - 1) / bs; }
inline int grid_of(const Geo& g) { return g.grid; }
inline int stream_grid(int n) { return nblocks(n); }  // streaming kernels without reductions

// grid-stride loop over the sites of a kernel
#define TG_SITES(s, n) \
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < (n); s += gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------
// Device state of one CG solve.  Lives in device memory; all the scalar
// recurrences of CG run on the device so no iteration needs the host.
// ---------------------------------------------------------------------------
struct CgState {
  double rr;        // |r|^2 of the (recursive) residual
  double rr0;       // |b|^2
  double stop;      // stop when rr < stop
  double alpha, beta;
  double rr_true;   // |b - A x|^2 at the last reliable update (mixed)
  int iter, maxiter, status, done;
  int since_ru, ru_interval, n_ru, need_ru;
  int log_index;    // slot of the per-trajectory solve log, -1 for none
  int restart;      // mixed: the last reliable update found the FP32 residual off by > 10x
};

// Mixed precision: a reliable update also happens once |r|^2 has fallen by
// this factor since the last one (FP32 recursive residuals lose accuracy
// beyond about 1e-3 in |r|), besides every ru_interval iterations.
constexpr double kRuDrop = 1e-6;
// ... and p restarts from r when the true |r|^2 exceeds the recursive one by this factor.
constexpr double kRuRestart = 10.0;

// Per-solve record kept for the host (iterations, status, reliable updates).
struct CgLog {
  int iter, status, n_ru, pad_;
  double rr, rr0;
};

// Graph conditional handles a CG kernel may set; use == 0 outside graphs.
struct Cond {
  cudaGraphConditionalHandle loop;   // WHILE node of the solve
  cudaGraphConditionalHandle ru;     // IF node of the reliable update (mixed)
  int use;
};

}  // namespace tg
