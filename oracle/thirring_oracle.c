/*
 * thirring_oracle.c -- CPU restatement of the Thirring2D HMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it.  No product code path links or calls it.
 *
 * It restates, from the mathematics, the algorithm of rantahar/Thirring2D
 * hmc.c with run-time lattice sizes, boundary conditions and mu (the
 * reference fixes NT/NX at compile time and caches exp(+-mu) in statics).
 * Every function cites the reference lines it follows.  Pinned against the
 * reference itself by tests/golden/ (fixtures produced by a patched build of
 * hmc.c, see oracle/make_ref.py).
 *
 * Conventions (same as the CUDA library):
 *   site index        s = t*nx + x          (hmc.c loops t outer, x inner)
 *   gauge field       A[2*s + dir], dir 0 = t, 1 = x   (hmc.c A[t][x][dir])
 *   fermion vectors   double complex v[s]             (hmc.c v[t][x])
 *   staggered phases  eta_t(x) = (-1)^x, eta_x = 1     (hmc.c:914-921)
 *   boundary signs    bc_t, bc_x in {+1,-1}; the hop across the last slice
 *                     picks up the sign (hmc.c:143-148, 165-170).  The
 *                     reference ships bc_t = bc_x = -1.
 *   adjoint           M^dagger is the true adjoint of M.  hmc.c:188-249
 *                     ships fm_conjugate_mul identical to fm_mul, which makes
 *                     its CG diverge; the oracle implements M^dagger.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846264338327
#endif

#define ORC_NF 2 /* hmc.c:28 */

typedef struct {
  int nt, nx;
  double m, g, mu;
  int bc_t, bc_x;
} orc_lattice;

/* ------------------------------------------------------------------ */
/* Random numbers: MT19937 with Knuth-69069 seeding and reverse block  */
/* consumption, as mersenne_inline.c:73-128 and mersenne.h:11 use it.  */
/* Algorithm: Matsumoto & Nishimura, ACM TOMACS 8 (1998) 3-30.         */
/* ------------------------------------------------------------------ */
typedef struct {
  uint32_t state[624];
  double block[624];
  int left; /* values of block[] not yet consumed; consumed from the top */
} orc_mt;

void orc_mt_seed(orc_mt* g, long seed) {
  /* mersenne_inline.c:73-87: odd seed, then x_{k} = 69069 x_{k-1} mod 2^32 */
  if (seed % 2 == 0) seed++;
  g->state[0] = (uint32_t)(seed & 0xffffffffL);
  for (int k = 1; k < 624; k++) g->state[k] = 69069u * g->state[k - 1];
  g->left = 0;
}

static void orc_mt_refill(orc_mt* g) {
  /* mersenne_inline.c:103-125: one twist of the 624-word state, then
   * tempering; each word becomes y * 2^-32 in [0,1). */
  uint32_t* s = g->state;
  for (int k = 0; k < 624; k++) {
    uint32_t y = (s[k] & 0x80000000u) | (s[(k + 1) % 624] & 0x7fffffffu);
    uint32_t v = s[(k + 397) % 624] ^ (y >> 1);
    if (y & 1u) v ^= 0x9908b0dfu;
    s[k] = v;
  }
  for (int k = 0; k < 624; k++) {
    uint32_t y = s[k];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    g->block[k] = ldexp((double)y, -32);
  }
  g->left = 624;
}

double orc_mt_next(orc_mt* g) {
  /* mersenne.h:11 hands out block[623], block[622], ... block[0] */
  if (g->left <= 0) orc_mt_refill(g);
  return g->block[--g->left];
}

void orc_mt_fill(orc_mt* g, double* out, long n) {
  for (long k = 0; k < n; k++) out[k] = orc_mt_next(g);
}

size_t orc_mt_sizeof(void) { return sizeof(orc_mt); }

/* Box-Muller pair from two consecutive draws, hmc.c:423-426, 488-491. */
static void orc_gauss_pair(orc_mt* g, double* re, double* im) {
  double u1 = orc_mt_next(g);
  double u2 = orc_mt_next(g);
  double r = sqrt(-2 * log(u1));
  *re = r * cos(2 * M_PI * u2);
  *im = r * sin(2 * M_PI * u2);
}

/* Complex Gaussian field, one pair per site in t-major order
 * (hmc.c:422-430, 441-446).  Returns sum |v|^2 (hmc.c:428). */
double orc_gaussian_field(orc_mt* g, int volume, double complex* v) {
  double s = 0;
  for (int k = 0; k < volume; k++) {
    double re, im;
    orc_gauss_pair(g, &re, &im);
    v[k] = re + I * im;
    s += re * re + im * im;
  }
  return s;
}

/* Momentum field, one pair per site: p_t = cos part, p_x = sin part
 * (hmc.c:486-495).  Returns sum p^2 (no 1/2, hmc.c:493). */
double orc_random_momentum(orc_mt* g, int volume, double* p) {
  double s = 0;
  for (int k = 0; k < volume; k++) {
    double re, im;
    orc_gauss_pair(g, &re, &im);
    p[2 * k] = re;
    p[2 * k + 1] = im;
    s += re * re + im * im;
  }
  return s;
}

/* ------------------------------------------------------------------ */
/* Geometry                                                            */
/* ------------------------------------------------------------------ */
static inline int eta_t(int x) { return (x % 2 == 0) ? 1 : -1; } /* hmc.c:917-921 */

/* Hopping coefficient of the link (s, s+dir): 0.5*eta*bc*exp(i A).  The
 * boundary sign is the one hmc.c applies when the forward neighbour wraps
 * (hmc.c:143-148 for t, 165-170 for x). */
static inline double complex link_coeff(const orc_lattice* L, const double* A, int t, int x, int dir) {
  int s = t * L->nx + x;
  double a = A[2 * s + dir];
  double sgn;
  if (dir == 0) sgn = eta_t(x) * ((t == L->nt - 1) ? L->bc_t : 1);
  else sgn = (x == L->nx - 1) ? L->bc_x : 1;
  return 0.5 * sgn * (cos(a) + I * sin(a));
}

/* ------------------------------------------------------------------ */
/* Fermion operator                                                    */
/* ------------------------------------------------------------------ */
/* M psi(s) = m psi(s) + e^{mu} W_t(s) psi(s+t) - e^{-mu} conj W_t(s-t) psi(s-t)
 *                     +        W_x(s) psi(s+x) -         conj W_x(s-x) psi(s-x)
 * which is hmc.c:132-183 term by term (mass 137, +t 140-148, -t 151-159,
 * +x 162-170, -x 172-180).  dagger=1 applies the true adjoint
 * M^dagger = m - D(-mu). */
void orc_apply(const orc_lattice* L, const double* A, const double complex* in, double complex* out, int dagger) {
  const int nt = L->nt, nx = L->nx;
  const double ep = exp(L->mu), em = exp(-L->mu);
  const double cf_t = dagger ? -em : ep;  /* forward t hop factor */
  const double cb_t = dagger ? ep : -em;  /* backward t hop factor */
  const double cf_x = dagger ? -1.0 : 1.0;
  const double cb_x = -cf_x;
  for (int t = 0; t < nt; t++) {
    int tu = (t + 1) % nt, td = (t - 1 + nt) % nt;
    for (int x = 0; x < nx; x++) {
      int xu = (x + 1) % nx, xd = (x - 1 + nx) % nx;
      int s = t * nx + x;
      double complex v = L->m * in[s];
      v += cf_t * link_coeff(L, A, t, x, 0) * in[tu * nx + x];
      v += cb_t * conj(link_coeff(L, A, td, x, 0)) * in[td * nx + x];
      v += cf_x * link_coeff(L, A, t, x, 1) * in[t * nx + xu];
      v += cb_x * conj(link_coeff(L, A, t, xd, 1)) * in[t * nx + xd];
      out[s] = v;
    }
  }
}

void orc_apply_M(const orc_lattice* L, const double* A, const double complex* in, double complex* out) {
  orc_apply(L, A, in, out, 0);
}
void orc_apply_Mdag(const orc_lattice* L, const double* A, const double complex* in, double complex* out) {
  orc_apply(L, A, in, out, 1);
}

/* Dense V x V matrix of M, row-major: (M psi)_i = sum_j Md[i*V+j] psi_j.
 * Same element set as hmc.c:269-310 (which stores it transposed for LAPACK). */
void orc_dense_M(const orc_lattice* L, const double* A, double complex* Md) {
  int V = L->nt * L->nx;
  double complex* e = calloc((size_t)V, sizeof(double complex));
  double complex* col = malloc((size_t)V * sizeof(double complex));
  for (int j = 0; j < V; j++) {
    e[j] = 1;
    orc_apply(L, A, e, col, 0);
    for (int i = 0; i < V; i++) Md[(size_t)i * V + j] = col[i];
    e[j] = 0;
  }
  free(e);
  free(col);
}

/* ------------------------------------------------------------------ */
/* Conjugate gradient on M^dagger M, hmc.c:341-404.                    */
/* Starts from x = 0.  Stops when |r|^2 < abs_tol2 (hmc.c:381, which   */
/* uses 1e-30) or |r|^2 < rel_tol^2 |b|^2 (rel_tol <= 0 disables).     */
/* Status: 0 converged, 1 max iterations (hmc.c:364 stops silently),   */
/* 2 diverged |r|^2/|r0|^2 > 1e10 (hmc.c:383-386 calls exit(1)), 3 NaN. */
/* ------------------------------------------------------------------ */
int orc_cg(const orc_lattice* L, const double* A, const double complex* b, double complex* x, double abs_tol2,
           double rel_tol, int maxiter, int* iters_out, double* rr_out) {
  int V = L->nt * L->nx;
  double complex* r = malloc((size_t)V * sizeof(double complex));
  double complex* p = malloc((size_t)V * sizeof(double complex));
  double complex* Mp = malloc((size_t)V * sizeof(double complex));
  double complex* MMp = malloc((size_t)V * sizeof(double complex));
  double rr = 0;
  for (int s = 0; s < V; s++) {
    x[s] = 0;
    r[s] = b[s];
    p[s] = b[s];
    rr += creal(r[s]) * creal(r[s]) + cimag(r[s]) * cimag(r[s]);
  }
  double rr0 = rr;
  double stop = abs_tol2;
  if (rel_tol > 0 && rel_tol * rel_tol * rr0 > stop) stop = rel_tol * rel_tol * rr0;
  int status = 0, k = 0;
  if (rr0 >= stop) {
    status = 1;
    for (k = 1; k <= maxiter; k++) {
      orc_apply(L, A, p, Mp, 0);
      orc_apply(L, A, Mp, MMp, 1);
      double pAp = 0;
      for (int s = 0; s < V; s++) pAp += creal(p[s]) * creal(MMp[s]) + cimag(p[s]) * cimag(MMp[s]);
      double a = rr / pAp;
      for (int s = 0; s < V; s++) x[s] += a * p[s];
      for (int s = 0; s < V; s++) r[s] -= a * MMp[s];
      double rn = 0;
      for (int s = 0; s < V; s++) rn += creal(r[s]) * creal(r[s]) + cimag(r[s]) * cimag(r[s]);
      if (isnan(rn)) { status = 3; rr = rn; break; }
      if (rn < stop) { status = 0; rr = rn; break; }
      if (rn / rr0 > 1e10) { status = 2; rr = rn; break; }
      double beta = rn / rr;
      for (int s = 0; s < V; s++) p[s] = r[s] + beta * p[s];
      rr = rn;
    }
    if (k > maxiter) k = maxiter;
  }
  if (iters_out) *iters_out = k;
  if (rr_out) *rr_out = rr;
  free(r); free(p); free(Mp); free(MMp);
  return status;
}

/* ------------------------------------------------------------------ */
/* Actions                                                             */
/* ------------------------------------------------------------------ */
/* S_g = (Nf/g) sum (1 - cos A), hmc.c:73-79 */
double orc_gauge_action(const orc_lattice* L, const double* A) {
  double S = 0;
  int n = 2 * L->nt * L->nx;
  for (int k = 0; k < n; k++) S += 1. - cos(A[k]);
  return ORC_NF / L->g * S;
}

/* Re <u, v> */
static double re_dot(int V, const double complex* u, const double complex* v) {
  double s = 0;
  for (int k = 0; k < V; k++) s += creal(u[k]) * creal(v[k]) + cimag(u[k]) * cimag(v[k]);
  return s;
}

/* S_md = Re <chi, M^dagger chi>, hmc.c:467-479 */
double orc_md_action(const orc_lattice* L, const double* A, const double complex* chi) {
  int V = L->nt * L->nx;
  double complex* tmp = malloc((size_t)V * sizeof(double complex));
  orc_apply(L, A, chi, tmp, 1);
  double s = re_dot(V, chi, tmp);
  free(tmp);
  return s;
}

/* S_pf = Re <phi, (M^dagger M)^{-1} phi>, hmc.c:451-463.  Returns CG status. */
int orc_pf_action(const orc_lattice* L, const double* A, const double complex* phi, double abs_tol2, double rel_tol,
                  int maxiter, double* S, int* iters) {
  int V = L->nt * L->nx;
  double complex* x = malloc((size_t)V * sizeof(double complex));
  int st = orc_cg(L, A, phi, x, abs_tol2, rel_tol, maxiter, iters, NULL);
  *S = re_dot(V, phi, x);
  free(x);
  return st;
}

/* ------------------------------------------------------------------ */
/* Leapfrog pieces                                                     */
/* ------------------------------------------------------------------ */
/* A += 2 eps p, hmc.c:97-101 (H has sum p^2, no 1/2) */
void orc_gauge_step(const orc_lattice* L, double* A, const double* p, double eps) {
  int n = 2 * L->nt * L->nx;
  for (int k = 0; k < n; k++) A[k] += 2.0 * eps * p[k];
}

/* Pseudofermion force on every link from chi = (M^dagger M)^{-1} phi and
 * Mchi = M chi, accumulated into F (dS_pf/dA).  Restates hmc.c:517-576:
 * dS/dA_mu(s) = 2 Im W (e^{mu} conj(Mchi(s)) chi(s+mu) - e^{-mu} conj(chi(s)) Mchi(s+mu))
 * with W = 0.5 eta bc e^{iA}, e^{+-mu} only on t links. */
void orc_pf_force(const orc_lattice* L, const double* A, const double complex* chi, const double complex* Mchi,
                  double* F) {
  const int nt = L->nt, nx = L->nx;
  const double ep = exp(L->mu), em = exp(-L->mu);
  for (int t = 0; t < nt; t++)
    for (int x = 0; x < nx; x++) {
      int s = t * nx + x;
      int su[2] = {((t + 1) % nt) * nx + x, t * nx + (x + 1) % nx};
      for (int dir = 0; dir < 2; dir++) {
        double complex W = link_coeff(L, A, t, x, dir);
        double e1 = dir == 0 ? ep : 1.0, e2 = dir == 0 ? em : 1.0;
        double complex c = e1 * conj(Mchi[s]) * chi[su[dir]] - e2 * conj(chi[s]) * Mchi[su[dir]];
        F[2 * s + dir] += 2.0 * cimag(W * c);
      }
    }
}

/* Force of the stochastic term Re <n, M^dagger n> (hmc.c:608-661).  Only t
 * links carry e^{+-mu}; x links get exactly zero (hmc.c:647-660, whose
 * st[t2][x] typo multiplies a zero).  Accumulated into F. */
void orc_md_force(const orc_lattice* L, const double* A, const double complex* n, double* F) {
  const int nt = L->nt, nx = L->nx;
  const double d = exp(L->mu) - exp(-L->mu);
  if (d == 0) return;
  for (int t = 0; t < nt; t++)
    for (int x = 0; x < nx; x++) {
      int s = t * nx + x;
      int su = ((t + 1) % nt) * nx + x;
      double complex W = link_coeff(L, A, t, x, 0);
      F[2 * s] += -d * cimag(W * conj(n[s]) * n[su]);
    }
}

/* Full dS/dA (gauge + pseudofermions + stochastic term) for npf solved
 * pseudofermions chi[k] with Mchi[k] = M chi[k]. */
void orc_total_force(const orc_lattice* L, const double* A, int npf, const double complex* chi,
                     const double complex* Mchi, const double complex* noise, double* F) {
  int V = L->nt * L->nx;
  for (int k = 0; k < 2 * V; k++) F[k] = ORC_NF / L->g * sin(A[k]); /* hmc.c:507-510 */
  for (int q = 0; q < npf; q++) orc_pf_force(L, A, chi + (size_t)q * V, Mchi + (size_t)q * V, F);
  if (noise) orc_md_force(L, A, noise, F);
}

/* momentum_step of hmc.c:504-665: p -= eps*(Nf/g) sin A on every link
 * (507-510), then per pseudofermion one CG and p -= eps*F_pf (515-576),
 * then p -= eps*F_md (608-661) -- the same three subtractions, in the same
 * order, as the reference.  Returns the largest CG status seen; iteration
 * counts are added to *iters. */
int orc_momentum_step(const orc_lattice* L, const double* A, double* p, int npf, const double complex* phi,
                      const double complex* noise, double eps, double abs_tol2, double rel_tol, int maxiter,
                      int* iters) {
  int V = L->nt * L->nx;
  double complex* chi = malloc((size_t)V * sizeof(double complex));
  double complex* Mchi = malloc((size_t)V * sizeof(double complex));
  double* F = malloc((size_t)2 * V * sizeof(double));
  int worst = 0;
  for (int k = 0; k < 2 * V; k++) p[k] -= eps * ORC_NF / L->g * sin(A[k]);
  for (int q = 0; q < npf; q++) {
    int it = 0;
    int st = orc_cg(L, A, phi + (size_t)q * V, chi, abs_tol2, rel_tol, maxiter, &it, NULL);
    if (st > worst) worst = st;
    if (iters) *iters += it;
    orc_apply(L, A, chi, Mchi, 0);
    memset(F, 0, (size_t)2 * V * sizeof(double));
    orc_pf_force(L, A, chi, Mchi, F);
    for (int k = 0; k < 2 * V; k++) p[k] -= eps * F[k];
  }
  if (noise) {
    memset(F, 0, (size_t)2 * V * sizeof(double));
    orc_md_force(L, A, noise, F);
    for (int k = 0; k < 2 * V; k++) p[k] -= eps * F[k];
  }
  free(chi); free(Mchi); free(F);
  return worst;
}

/* ------------------------------------------------------------------ */
/* One HMC trajectory, hmc.c:671-746, with the random numbers drawn   */
/* from the MT stream in the reference order: pseudofermion pairs      */
/* (hmc.c:695), momentum pairs (696), noise pairs (698), accept (738). */
/* stats[0..9] = dH, Sg0, Spf0, Smd0, Smom0, Sg1, Spf1, Smd1, Smom1,  */
/* accepted.  Returns the worst CG status; *cg_iters sums iterations.  */
/* ------------------------------------------------------------------ */
int orc_trajectory(const orc_lattice* L, double* A, orc_mt* g, int nsteps, double tau, int npf, int use_noise,
                   double abs_tol2, double rel_tol, int maxiter, double* stats, int* cg_iters) {
  int V = L->nt * L->nx;
  double complex* eta = malloc((size_t)V * sizeof(double complex));
  double complex* phi = malloc((size_t)npf * V * sizeof(double complex));
  double complex* noise = malloc((size_t)V * sizeof(double complex));
  double* p = malloc((size_t)2 * V * sizeof(double));
  double* An = malloc((size_t)2 * V * sizeof(double));
  int worst = 0, it = 0;
  double Spf0 = 0;
  for (int q = 0; q < npf; q++) {
    Spf0 += orc_gaussian_field(g, V, eta);   /* hmc.c:418-436 */
    orc_apply(L, A, eta, phi + (size_t)q * V, 1);
  }
  double Smom0 = orc_random_momentum(g, V, p);
  double Sg0 = orc_gauge_action(L, A);
  double Smd0 = 0;
  if (use_noise) {
    orc_gaussian_field(g, V, noise);
    Smd0 = orc_md_action(L, A, noise);
  }
  memcpy(An, A, (size_t)2 * V * sizeof(double));
  double eps = tau / nsteps;
  for (int i = 0; i < nsteps; i++) {                     /* hmc.c:710-716 */
    orc_gauge_step(L, An, p, tau * 0.5 / nsteps);
    int st = orc_momentum_step(L, An, p, npf, phi, use_noise ? noise : NULL, eps, abs_tol2, rel_tol, maxiter, &it);
    if (st > worst) worst = st;
    orc_gauge_step(L, An, p, tau * 0.5 / nsteps);
  }
  double Spf1 = 0;
  for (int q = 0; q < npf; q++) {
    double s; int i2 = 0;
    int st = orc_pf_action(L, An, phi + (size_t)q * V, abs_tol2, rel_tol, maxiter, &s, &i2);
    if (st > worst) worst = st;
    it += i2;
    Spf1 += s;
  }
  double Smom1 = 0;
  for (int k = 0; k < 2 * V; k++) Smom1 += p[k] * p[k];
  double Sg1 = orc_gauge_action(L, An);
  double Smd1 = use_noise ? orc_md_action(L, An, noise) : 0;
  double dS = Smom1 - Smom0 + Spf1 - Spf0 + Smd1 - Smd0 + Sg1 - Sg0; /* hmc.c:729-732 */
  int acc = exp(-dS) > orc_mt_next(g);                                /* hmc.c:738 */
  if (acc) memcpy(A, An, (size_t)2 * V * sizeof(double));
  double out[10] = {dS, Sg0, Spf0, Smd0, Smom0, Sg1, Spf1, Smd1, Smom1, (double)acc};
  memcpy(stats, out, sizeof(out));
  if (cg_iters) *cg_iters = it;
  free(eta); free(phi); free(noise); free(p); free(An);
  return worst;
}

/* Pure-gauge Metropolis sweep, hmc.c:82-93: propose A' = 2 pi u - pi,
 * accept if u' < exp(-(S(A') - S(A))).  Two draws per link. */
void orc_puregauge_sweep(const orc_lattice* L, double* A, orc_mt* g) {
  int n = 2 * L->nt * L->nx;
  for (int k = 0; k < n; k++) {
    double s1 = -ORC_NF / L->g * cos(A[k]);
    double a = 2 * M_PI * orc_mt_next(g) - M_PI;
    double s2 = -ORC_NF / L->g * cos(a);
    double w = exp(-s2 + s1);
    if (orc_mt_next(g) < w) A[k] = a;
  }
}

/* ------------------------------------------------------------------ */
/* Secondary rows: the real, A-free, monomer-masked operator of the    */
/* fermion-bag programs (vec_ops.c:96-174, ANTISYMMETRIC/OPENX build)  */
/* and CG on fM^T fM (vec_ops.c:261-307).  mask[s] != 0 marks an       */
/* occupied site: its row is the identity and it is skipped as a       */
/* neighbour.  bc_t/bc_x as above (the ANTISYMMETRIC build uses -1,-1). */
/* ------------------------------------------------------------------ */
void orc_fM(const orc_lattice* L, const int* mask, const double* in, double* out, int transpose) {
  const int nt = L->nt, nx = L->nx;
  const double ep = exp(L->mu), em = exp(-L->mu);
  /* fM: +t hop e^{mu}, -t hop e^{-mu}, both with +eta (vec_ops.c:109-118);
   * fM_transpose negates the hops and swaps e^{+-mu} (vec_ops.c:148-157). */
  const double sg = transpose ? -1.0 : 1.0;
  const double fu = transpose ? em : ep, fd = transpose ? ep : em;
  for (int t = 0; t < nt; t++)
    for (int x = 0; x < nx; x++) {
      int s = t * nx + x;
      if (mask[s]) { out[s] = in[s]; continue; }
      double v = L->m * in[s];
      int tu = (t + 1) % nt, td = (t - 1 + nt) % nt, xu = (x + 1) % nx, xd = (x - 1 + nx) % nx;
      double et = eta_t(x);
      /* forward neighbour: + unless the hop wraps (then bc); backward: + only
       * when the hop wraps (t2 > t branch), else - */
      if (!mask[tu * nx + x]) v += sg * 0.5 * et * fu * (tu > t ? 1.0 : L->bc_t) * in[tu * nx + x];
      if (!mask[td * nx + x]) v += sg * 0.5 * et * fd * (td > t ? -L->bc_t : -1.0) * in[td * nx + x];
      if (!mask[t * nx + xu]) v += sg * 0.5 * (xu > x ? 1.0 : L->bc_x) * in[t * nx + xu];
      if (!mask[t * nx + xd]) v += sg * 0.5 * (xd > x ? -L->bc_x : -1.0) * in[t * nx + xd];
      out[s] = v;
    }
}

/* vec_ops.c:261-307: CG on fM^T fM from 0; stops at |r|^2 < abs_tol2 or
 * rel_tol; on divergence the reference fills the result with 1e50 and
 * returns -- here status 2 is returned instead. */
int orc_cg_MdM(const orc_lattice* L, const int* mask, const double* b, double* xo, double abs_tol2, double rel_tol,
               int maxiter, int* iters_out) {
  int V = L->nt * L->nx;
  double* r = malloc((size_t)V * sizeof(double));
  double* p = malloc((size_t)V * sizeof(double));
  double* Mp = malloc((size_t)V * sizeof(double));
  double* MMp = malloc((size_t)V * sizeof(double));
  double rr = 0;
  for (int s = 0; s < V; s++) { xo[s] = 0; r[s] = p[s] = b[s]; rr += b[s] * b[s]; }
  double rr0 = rr, stop = abs_tol2;
  if (rel_tol > 0 && rel_tol * rel_tol * rr0 > stop) stop = rel_tol * rel_tol * rr0;
  int status = 0, k = 0;
  if (rr0 >= stop) {
    status = 1;
    for (k = 1; k <= maxiter; k++) {
      orc_fM(L, mask, p, Mp, 0);
      orc_fM(L, mask, Mp, MMp, 1);
      double pAp = 0;
      for (int s = 0; s < V; s++) pAp += p[s] * MMp[s];
      double a = rr / pAp;
      for (int s = 0; s < V; s++) { xo[s] += a * p[s]; r[s] -= a * MMp[s]; }
      double rn = 0;
      for (int s = 0; s < V; s++) rn += r[s] * r[s];
      if (isnan(rn)) { status = 3; break; }
      if (rn < stop) { status = 0; break; }
      if (rn / rr0 > 1e10) { status = 2; break; }
      double beta = rn / rr;
      for (int s = 0; s < V; s++) p[s] = r[s] + beta * p[s];
      rr = rn;
    }
    if (k > maxiter) k = maxiter;
  }
  if (iters_out) *iters_out = k;
  free(r); free(p); free(Mp); free(MMp);
  return status;
}
