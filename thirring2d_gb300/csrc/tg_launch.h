// tg_launch.h -- host-side launch interface between tg_kernels.cu and tg_capi.cu.
#pragma once

#include "tg_internal.cuh"

namespace tg {

// Per-trajectory scalars on the device (filled by the reduction kernels).
struct TrajStats {
  double Sg0, Spf0, Smd0, Smom0;
  double Sg1, Spf1, Smd1, Smom1;
  double dH, u;
  int accepted, pad_;
  unsigned long long traj;   // Philox trajectory counter
};

struct CgBufs64 {          // FP64 CG work vectors (p alternates between two buffers)
  double2 *r, *p[2], *Mp;
};
struct CgBufsMixed {       // FP32 CG work vectors + FP64 accumulators
  float2 *xs, *rs, *ps[2], *Mps;
  double2* tmp64;          // M x for the reliable update
  float2* ss;              // single-reduction CG: s (its w is Mps, p ps[0], r rs)
};

struct Red {               // reduction scratch
  double* partials;
  unsigned* counter;
};

struct Links {
  const double2 *Wt, *Wx;
  const float2 *Wt32, *Wx32;
  // W / m and 1 / m^2 for the unit-mass form of the FP64 CG (null when m = 0)
  const double2 *Wt1 = nullptr, *Wx1 = nullptr;
  double inv_m2 = 0;
};

// Where the link kernels write: W (FP64, FP32) and, when Wt1 is non-null, W / m
struct LinkOut {
  double2 *Wt, *Wx;
  float2 *Wt32, *Wx32;
  double2 *Wt1 = nullptr, *Wx1 = nullptr;
  double inv_m = 0;
};

// link coefficients of A (both precisions)
void link_phase(cudaStream_t s, const Geo& g, int bc_t, int bc_x, const double2* A, const LinkOut& o);
// A += c*mom, nadd times in sequence, then link coefficients
void gauge_step(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double2* A, const double2* mom, double c,
                int nadd, const LinkOut& o);
// out = M in (dag = 0) or M^dag in (dag = 1); k must be the constants of that operator
void dslash64(cudaStream_t s, const Geo& g, const OpK<double>& k, int dag, const double2* in, double2* out,
              const double2* Wt, const double2* Wx);
void dslash32(cudaStream_t s, const Geo& g, const OpK<float>& k, int dag, const float2* in, float2* out,
              const float2* Wt, const float2* Wx);

// CG on M^dag M (FP64).  km = M constants, kd = M^dag constants.
void cg64_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufs64& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int log_index, Cond c);
// one iteration reading p[half] and writing p[half ^ 1]; iterations alternate half = 0, 1
void cg64_iter(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
               double2* x, const CgBufs64& w, int half, CgState* st, CgLog* log, const Red& red, Cond c);
// Mixed precision: FP32 iterations + FP64 reliable update
void cgmx_init(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufsMixed& w, CgState* st,
               CgLog* log, const Red& red, double rel_tol, double abs_tol2, int maxiter, int ru_interval,
               int log_index, Cond c);
void cgmx_iter(cudaStream_t s, const Geo& g, const OpK<float>& km, const OpK<float>& kd, const Links& L,
               const CgBufsMixed& w, int half, CgState* st, const Red& red, Cond c);
void cgmx_reliable(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
                   const double2* b, double2* x, const CgBufsMixed& w, CgState* st, CgLog* log, const Red& red,
                   Cond c);

// reductions into a device double (accumulate: *dst += sum, else *dst = sum)
void norm2(cudaStream_t s, const Geo& g, const double2* v, double* dst, int accumulate, const Red& red);
void redot(cudaStream_t s, const Geo& g, const double2* u, const double2* v, double* dst, int accumulate,
           const Red& red);
void gauge_action(cudaStream_t s, const Geo& g, const double2* A, double fac, double* dst, const Red& red);
void md_action(cudaStream_t s, const Geo& g, const OpK<double>& kd, const double2* nz, const double2* Wt,
               const double2* Wx, double* dst, const Red& red);

// mom -= eps*F; flags bit0: gauge force first (gfac = eps*Nf/g), bit1: stochastic-term force last
// (bc_t, bc_x: the lattice's boundary conditions, which the link coefficients carry)
void momentum_update(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double ep, double em, const double2* A,
                     const double2* Wt, const double2* Wx, const double2* chi, const double2* Mchi,
                     const double2* noise, double2* mom, double eps, double gfac, int flags);
// F = dS/dA (for tests): same pieces, written instead of applied
void force_field(cudaStream_t s, const Geo& g, int bc_t, int bc_x, double ep, double em, const double2* A,
                 const double2* Wt, const double2* Wx, const double2* chi, const double2* Mchi, const double2* noise,
                 double2* F, double gfac, int flags);

// Philox Gaussian fields: out[n] complex pairs for (seed, stats->traj, stream_id)
void philox_gauss(cudaStream_t s, const Geo& g, unsigned long long seed, const TrajStats* ts, unsigned stream_id,
                  double2* out);
void philox_uniform(cudaStream_t s, unsigned long long seed, TrajStats* ts, unsigned stream_id);

void finish_trajectory(cudaStream_t s, TrajStats* ts);
void accept_copy(cudaStream_t s, const Geo& g, const TrajStats* ts, double2* A, const double2* Anew);
// one pure-gauge Metropolis sweep over the 2V links; u[4V]; c = -Nf/g
void puregauge(cudaStream_t s, const Geo& g, double* A, const double* u, double c);

// Measurements and the masked real operator (tg_aux.cu)
void sum_links(cudaStream_t s, const Geo& g, const double2* A, double* dst, const Red& red);
void imdot(cudaStream_t s, const Geo& g, const double2* u, const double2* v, double* dst, int acc, const Red& red);
void fm_apply(cudaStream_t s, const Geo& g, double m, double mu, int bc_t, int bc_x, const int* mask,
              const double* in, double* out, int transpose);
void rcg_init(cudaStream_t s, const Geo& g, const double* b, double* x, double* r, double* p, double rel_tol,
              double abs_tol2, int maxiter, CgState* st, const Red& red);
void rcg_iter(cudaStream_t s, const Geo& g, double m, double mu, int bc_t, int bc_x, const int* mask, double* x,
              double* r, double* p, double* tmp, double* Ap, CgState* st, const Red& red);

void dense_M(cudaStream_t s, const Geo& g, const OpK<double>& k, const double2* Wt, const double2* Wx, double2* Md);
// log|det| and arg det of nmat V x V complex matrices (overwritten by their LU factors)
void lu_logdet(cudaStream_t s, int V, int nmat, double2* mats, double* out);

// ---------------------------------------------------------------------------
// Persistent CG (tg_pcg.cu): one cooperative launch per solve
// ---------------------------------------------------------------------------
// The persistent solver's barrier words, all 0 at launch: the arrival count,
// a spare word, then the two 64-bit words of the fixed-point sums (one per
// kind of iteration sum of the mixed CG; see tg_pcg.cu).
constexpr int kBarWords = 6;
struct GridBar {
  unsigned* count;           // grid barrier: monotonic arrival count
  unsigned long long* fx;    // fixed-point sums: 2 words (count + 2)
};
// largest persistent grid; partial sums: 4 * kPcgMaxGrid doubles (two alternating
// arrays of (gamma, delta) pairs in the single-reduction CG)
constexpr int kPcgMaxGrid = 4096;

struct Pcg64Args {
  Geo g;
  OpK<double> km, kd;
  const double2 *Wt, *Wx;  // W, or W / m with inv_m2 = 1 / m^2 (unit-mass form); inv_m2 = 0: plain
  double inv_m2;
  const double2* b;
  double2 *x, *r, *p0, *p1, *Mp;
  CgState* st;
  CgLog* log;
  int log_index;
  double* part;
  GridBar bar;
  double rel_tol, abs_tol2;
  int maxiter;
};

struct PcgMxArgs {
  Geo g;
  OpK<float> km32, kd32;
  OpK<double> km, kd;
  const float2 *Wt32, *Wx32;
  const double2 *Wt, *Wx;
  const double2* b;
  double2 *x, *tmp;
  float2 *xs, *r, *p0, *p1, *Mp;
  // single-reduction CG (k_pcgcg): w and s; p0 is p, r is r
  float2 *w0, *s0;
  CgState* st;
  CgLog* log;
  int log_index;
  double* part;
  GridBar bar;
  double rel_tol, abs_tol2;
  int maxiter, ru_interval;
};

cudaError_t pcg64(cudaStream_t s, bool mu0, Pcg64Args a);
cudaError_t pcgmx(cudaStream_t s, bool mu0, PcgMxArgs a);
// the mixed solve as a single-reduction CG (lattices with g.march only; same
// arguments and results): per iteration an elementwise update and one pass of
// the fused M^dag M march (k_pcgcg)
cudaError_t pcgcg(cudaStream_t s, bool mu0, PcgMxArgs a);
// one grid barrier (4 blocks, cooperative) that also waits for `phantom` absent
// blocks, giving up after `limit` polls: *status = TG_OK or TG_E_TIMEOUT
cudaError_t barrier_check(cudaStream_t s, unsigned* count, unsigned phantom, long long limit, int* status);

// staged-kernel waits (tg_kernels.cu) that ran out since the library was loaded
unsigned stage_faults();

// Propagator matrix (calc_Dinv): one CG per source site, one block per source
struct PropArgs {
  Geo g;
  double m, ep, em;
  int bc_t, bc_x;
  const int* mask;
  int src0;         // first source site of this launch
  double* scratch;  // [sources of the launch][5][V]
  double* Dinv;     // [2][V/2][V/2]
  double abs_tol2, rel_tol;
  int maxiter;
  int* max_iter;    // atomicMax of the iterations of every source
  int* worst;       // atomicMax of the statuses
};
void prop_cg(cudaStream_t s, int nsrc, const PropArgs& a);

// FP64 FMA throughput probe: grid * 256 * 32 * iters FMAs, writes nothing
void dfma_peak(cudaStream_t s, int grid, int iters, double* sink);

// Explicit-grid launchers used by the allocation-free CG entry point.
int resident_grid_nocache(const void* kernel, int work);
void link_phase_fixed(cudaStream_t s, const Geo& g, int bc_t, int bc_x, const double2* A, double2* Wt, double2* Wx,
                      float2* Wt32, float2* Wx32);
void cg64_init_fixed(cudaStream_t s, const Geo& g, const double2* b, double2* x, const CgBufs64& w, CgState* st,
                     const Red& red, double rel_tol, double abs_tol2, int maxiter);
void cg64_iter_fixed(cudaStream_t s, const Geo& g, const OpK<double>& km, const OpK<double>& kd, const Links& L,
                     double2* x, const CgBufs64& w, int half, CgState* st, const Red& red);

}  // namespace tg
