/*
 * hmc_compat.c -- the function set of rantahar/Thirring2D hmc.c with its exact
 * names, signatures, globals and printed lines (include/thirring_hmc.h), run
 * on the GB300 library through its C ABI (include/thirring_gpu.h).
 *
 * The caller's row-pointer arrays (v[t][x], A[t][x][dir], as hmc.c:105-112 and
 * 888-898 allocate them) are gathered into contiguous host buffers, the work
 * is done on the device by one persistent tg_lattice, and results are
 * scattered back.  Random numbers come from the same MT19937 stream as
 * hmc.c's (the mersenne() macro of mersenne.h reads mersenne_i and
 * mersenne_array, defined here), consumed in the same order, so a program
 * that seeds it the same way draws the same fields.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "thirring_gpu.h"
#include "thirring_hmc.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846264338327
#endif

/* ---- globals of hmc.c:38-50 -------------------------------------------- */
double m;
double g;
double mu;
int *tup, *xup, *tdn, *xdn;
double*** A;
int*** eta;

/* ---- the MT19937 stream of mersenne_inline.c ---------------------------- */
int mersenne_i = -1;
double mersenne_array[MERSENNE_N];
static uint32_t mt_state[MERSENNE_N];

/* Knuth's 69069 recurrence from an odd seed (mersenne_inline.c:73-87). */
void seed_mersenne(long seed) {
  if (seed % 2 == 0) seed++;
  mt_state[0] = (uint32_t)(seed & 0xffffffffL);
  for (int k = 1; k < MERSENNE_N; k++) mt_state[k] = 69069u * mt_state[k - 1];
  mersenne_i = 0;
}

/* One MT19937 twist (Matsumoto & Nishimura 1998) and tempering into
 * mersenne_array; hands out the last element first (mersenne_inline.c:89-128). */
double mersenne_generate(void) {
  if (mersenne_i < 0) {
    printf("DUMMY: you did not seed the generator!\n");
    exit(0);
  }
  for (int k = 0; k < MERSENNE_N; k++) {
    uint32_t y = (mt_state[k] & 0x80000000u) | (mt_state[(k + 1) % MERSENNE_N] & 0x7fffffffu);
    uint32_t v = mt_state[(k + 397) % MERSENNE_N] ^ (y >> 1);
    mt_state[k] = (y & 1u) ? (v ^ 0x9908b0dfu) : v;
  }
  for (int k = 0; k < MERSENNE_N; k++) {
    uint32_t y = mt_state[k];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    mersenne_array[k] = (double)y * (1.0 / 4294967296.0);
  }
  mersenne_i = MERSENNE_N;
  return mersenne_array[--mersenne_i];
}

/* Box-Muller pair as hmc.c:423-426 */
static void gauss_pair(double* re, double* im) {
  double u1 = mersenne();
  double u2 = mersenne();
  double r = sqrt(-2 * log(u1));
  *re = r * cos(2 * M_PI * u2);
  *im = r * sin(2 * M_PI * u2);
}

/* ---- the device lattice behind the globals ----------------------------- */
static int NT_ = 0, NX_ = 0;
static tg_lattice* lat = NULL;
static double cur_m, cur_g, cur_mu;
static double *fa, *fb, *fc, *fd; /* contiguous host buffers, 2*V doubles each */

void thirring_hmc_set_lattice(int nt, int nx) {
  if (lat) {
    tg_destroy(lat);
    lat = NULL;
  }
  NT_ = nt;
  NX_ = nx;
}

static int env_int(const char* name, int dflt) {
  const char* e = getenv(name);
  return e ? atoi(e) : dflt;
}

int thirring_hmc_nt(void) {
  if (!NT_) NT_ = env_int("HMC_NT", 32);
  return NT_;
}
int thirring_hmc_nx(void) {
  if (!NX_) NX_ = env_int("HMC_NX", 32);
  return NX_;
}

static void fatal(const char* where) {
  fprintf(stderr, "thirring_hmc: %s: %s\n", where, tg_last_error());
  exit(1);
}

/* Solver statuses follow hmc.c: divergence prints its message and exits
 * (hmc.c:383-386); the iteration cap stops silently (hmc.c:364). */
static void check(int rc, const char* where) {
  if (rc == TG_OK || rc == TG_E_NOCONV) return;
  if (rc == TG_E_DIVERGED || rc == TG_E_NAN) {
    printf("Cannot invert fermion matrix\n");
    exit(1);
  }
  fatal(where);
}

static tg_lattice* ctx(void) {
  int nt = thirring_hmc_nt(), nx = thirring_hmc_nx();
  if (!lat) {
    const char* bc = getenv("HMC_BC_X");
    tg_lattice_params p;
    memset(&p, 0, sizeof p);
    p.nt = nt;
    p.nx = nx;
    p.m = m;
    p.g = g > 0 ? g : 1.0;
    p.mu = mu;
    p.bc_t = TG_BC_ANTIPERIODIC;
    p.bc_x = (bc && strcmp(bc, "periodic") == 0) ? TG_BC_PERIODIC : TG_BC_ANTIPERIODIC;
    p.device = env_int("HMC_DEVICE", 0);
    if (tg_create(&p, &lat) != TG_OK) fatal("tg_create");
    size_t n = 2 * (size_t)nt * nx;
    free(fa); free(fb); free(fc); free(fd);
    fa = malloc(n * sizeof(double));
    fb = malloc(n * sizeof(double));
    fc = malloc(n * sizeof(double));
    fd = malloc(n * sizeof(double));
    cur_m = p.m; cur_g = p.g; cur_mu = p.mu;
  }
  if (m != cur_m || g != cur_g || mu != cur_mu) { /* hmc.c reads the globals at every call */
    if (tg_set_couplings(lat, m, g, mu) != TG_OK) fatal("tg_set_couplings");
    cur_m = m; cur_g = g; cur_mu = mu;
  }
  return lat;
}

static tg_cg_params cg_params(void) {
  tg_cg_params c;
  memset(&c, 0, sizeof c);
  const char* rel = getenv("HMC_CG_REL");
  const char* prec = getenv("HMC_PRECISION");
  c.rel_tol = rel ? atof(rel) : 0.0;
  c.abs_tol2 = rel ? 0.0 : 1e-30; /* hmc.c:34 */
  c.maxiter = 100000;             /* hmc.c:35 */
  c.precision = (prec && strcmp(prec, "mixed") == 0) ? TG_PREC_MIXED : TG_PREC_FP64;
  c.ru_interval = env_int("HMC_RU_INTERVAL", 50);
  return c;
}

/* row pointers <-> contiguous (t-major) */
static void gather_v(_Complex double** v, double* f) {
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      f[2 * (t * NX_ + x)] = creal(v[t][x]);
      f[2 * (t * NX_ + x) + 1] = cimag(v[t][x]);
    }
}
static void scatter_v(const double* f, _Complex double** v) {
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) v[t][x] = f[2 * (t * NX_ + x)] + I * f[2 * (t * NX_ + x) + 1];
}
static void gather_l(double*** a, double* f) {
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      f[2 * (t * NX_ + x)] = a[t][x][0];
      f[2 * (t * NX_ + x) + 1] = a[t][x][1];
    }
}
static void scatter_l(const double* f, double*** a) {
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      a[t][x][0] = f[2 * (t * NX_ + x)];
      a[t][x][1] = f[2 * (t * NX_ + x) + 1];
    }
}
static void upload_gauge(double*** a) {
  gather_l(a, fd);
  if (tg_set_gauge(ctx(), fd) != TG_OK) fatal("tg_set_gauge");
}

/* ---- hmc.c entry points ------------------------------------------------ */
_Complex double** alloc_vector(void) {
  int nt = thirring_hmc_nt(), nx = thirring_hmc_nx();
  _Complex double** v = malloc(nt * sizeof(_Complex double*));
  for (int t = 0; t < nt; t++) v[t] = malloc(nx * sizeof(_Complex double));
  return v;
}

void free_vector(_Complex double** v) {
  for (int t = 0; t < thirring_hmc_nt(); t++) free(v[t]);
  free(v);
}

static void apply(_Complex double** in, _Complex double** out, double*** a, int dagger) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_v(in, fa);
  if (tg_apply(L, fa, fb, dagger) != TG_OK) fatal("tg_apply");
  scatter_v(fb, out);
}

void fm_mul(_Complex double** v_in, _Complex double** v_out, double*** a) { apply(v_in, v_out, a, 0); }
void fm_conjugate_mul(_Complex double** v_in, _Complex double** v_out, double*** a) { apply(v_in, v_out, a, 1); }

void fmdm_invert_cg(_Complex double** v_in, _Complex double** v_out, double*** a) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_v(v_in, fa);
  tg_cg_params cp = cg_params();
  tg_cg_result r;
  check(tg_cg(L, &cp, fa, fb, &r), "tg_cg");
  scatter_v(fb, v_out);
}

/* hmc.c:408-414: x = (M^dag M)^-1 M^dag b = M^-1 b */
void fm_invert_cg(_Complex double** v_in, _Complex double** v_out, double*** a) {
  _Complex double** tmp = alloc_vector();
  fm_conjugate_mul(v_in, tmp, a);
  fmdm_invert_cg(tmp, v_out, a);
  free_vector(tmp);
}

double random_pseudofermion(_Complex double** v, double*** a) {
  ctx();
  double action = 0;
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      double re, im;
      gauss_pair(&re, &im);
      fc[2 * (t * NX_ + x)] = re;
      fc[2 * (t * NX_ + x) + 1] = im;
      action += re * re + im * im;
    }
  upload_gauge(a);
  if (tg_apply(lat, fc, fb, 1) != TG_OK) fatal("tg_apply");
  scatter_v(fb, v);
  return action;
}

void stochastic_vector(_Complex double** v) {
  ctx();
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      double re, im;
      gauss_pair(&re, &im);
      v[t][x] = re + I * im;
    }
}

double pseudofermion_action(_Complex double** v, double*** a) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_v(v, fa);
  tg_cg_params cp = cg_params();
  tg_cg_result r;
  double S = 0;
  check(tg_pseudofermion_action(L, &cp, fa, &S, &r), "tg_pseudofermion_action");
  return S;
}

double stochastic_md_action(_Complex double** v, double*** a) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_v(v, fa);
  double S = 0;
  if (tg_md_action(L, fa, &S) != TG_OK) fatal("tg_md_action");
  return S;
}

double random_momentum(double*** mom) {
  ctx();
  double action = 0;
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++) {
      double re, im;
      gauss_pair(&re, &im);
      mom[t][x][0] = re;
      mom[t][x][1] = im;
      action += re * re + im * im;
    }
  return action;
}

double momentum_step(double*** mom, double*** a, _Complex double** psi, _Complex double** st, double eps) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_l(mom, fc);
  gather_v(psi, fa);
  gather_v(st, fb);
  tg_cg_params cp = cg_params();
  tg_cg_result r;
  check(tg_momentum_step(L, &cp, fc, 1, fa, fb, eps, &r), "tg_momentum_step");
  scatter_l(fc, mom);
  return 0.0; /* declared double in hmc.c:504 but returns nothing */
}

double gauge_step(double*** a, double*** mom, double eps) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  gather_l(mom, fc);
  if (tg_gauge_step(L, fc, eps) != TG_OK) fatal("tg_gauge_step");
  if (tg_get_gauge(L, fd) != TG_OK) fatal("tg_get_gauge");
  scatter_l(fd, a);
  return 0.0; /* declared double in hmc.c:97 but returns nothing */
}

double calc_gauge_action(double*** a) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  double S = 0;
  if (tg_gauge_action(L, &S) != TG_OK) fatal("tg_gauge_action");
  return S;
}

void update_puregauge_hb(double*** a) {
  tg_lattice* L = ctx();
  size_t nl = 2 * (size_t)NT_ * NX_;
  double* u = malloc(2 * nl * sizeof(double));
  for (size_t k = 0; k < 2 * nl; k++) u[k] = mersenne(); /* hmc.c:85, 89: proposal, acceptance */
  upload_gauge(a);
  if (tg_puregauge_ext(L, u, 1) != TG_OK) fatal("tg_puregauge_ext");
  free(u);
  if (tg_get_gauge(L, fd) != TG_OK) fatal("tg_get_gauge");
  scatter_l(fd, a);
}

/* HMC_JSONL=<path>: one JSON line per trajectory appended to <path> (dH, the
 * actions, the decision, CG work and device time). */
static void log_trajectory(const tg_traj_result* r) {
  static FILE* fp = NULL;
  static int opened = 0;
  static long n = 0;
  if (!opened) {
    opened = 1;
    const char* path = getenv("HMC_JSONL");
    if (path && *path) fp = fopen(path, "a");
  }
  if (!fp) return;
  fprintf(fp,
          "{\"trajectory\": %ld, \"dH\": %.17g, \"Sg0\": %.17g, \"Spf0\": %.17g, \"Smd0\": %.17g, "
          "\"Smom0\": %.17g, \"Sg1\": %.17g, \"Spf1\": %.17g, \"Smd1\": %.17g, \"Smom1\": %.17g, "
          "\"u\": %.17g, \"accepted\": %d, \"cg_solves\": %d, \"cg_iterations\": %d, "
          "\"cg_max_iterations\": %d, \"reliable_updates\": %d, \"cg_ms\": %.6g}\n",
          ++n, r->dH, r->Sg0, r->Spf0, r->Smd0, r->Smom0, r->Sg1, r->Spf1, r->Smd1, r->Smom1, r->u_accept,
          r->accepted, r->cg_solves, r->cg_iterations, r->cg_max_iterations, r->reliable_updates, r->cg_ms);
  fflush(fp);
}

/* update_gauge, hmc.c:671-746: the random fields are drawn here from the
 * shared stream in hmc.c's order (pseudofermion, momentum, noise, then the
 * accept uniform -- nothing else draws in between), the trajectory runs on
 * the device, and A is replaced by the new field on acceptance. */
void update_gauge(double*** a) {
  tg_lattice* L = ctx();
  size_t V = (size_t)NT_ * NX_;
  double* f = malloc(6 * V * sizeof(double));
  for (size_t k = 0; k < 3 * V; k++) gauss_pair(&f[2 * k], &f[2 * k + 1]);
  double u = mersenne();
  upload_gauge(a);
  tg_hmc_params hp;
  memset(&hp, 0, sizeof hp);
  hp.nsteps = env_int("HMC_NSTEPS", 10); /* hmc.c:708 */
  hp.tau = 1.0;                         /* hmc.c:709 */
  hp.npf = 1;
  hp.stochastic_term = 1;
  hp.rng = TG_RNG_EXTERNAL;
  hp.use_graph = 1;
  hp.cg = cg_params();
  tg_traj_result r;
  check(tg_trajectory_ext(L, &hp, f, f + 2 * V, f + 4 * V, u, &r), "tg_trajectory_ext");
  free(f);
  /* HMC_VERBOSE=1: the same lines with every digit (%.17g) */
  const char* fmt0 = env_int("HMC_VERBOSE", 0) ? "Start HMC: Sg %.17g, Smdm %.17g, Smd %.17g, Smom %.17g\n"
                                               : "Start HMC: Sg %g, Smdm %g, Smd %g, Smom %g\n";
  const char* fmt1 = env_int("HMC_VERBOSE", 0) ? "HMC End, dS %.17g, Sg %.17g, Smdm %.17g, Smd %.17g, Sm %.17g\n"
                                               : "HMC End, dS %g, Sg %g, Smdm %g, Smd %g, Sm %g\n";
  printf(fmt0, r.Sg0, r.Spf0, r.Smd0, r.Smom0);
  printf(fmt1, r.dH, r.Sg1, r.Spf1, r.Smd1, r.Smom1);
  log_trajectory(&r);
  if (r.accepted) {
    printf("HMC ACCEPTED\n");
    if (tg_get_gauge(L, fd) != TG_OK) fatal("tg_get_gauge");
    scatter_l(fd, a);
  } else {
    printf("HMC REJECTED\n");
  }
}

/* hmc.c:269-310: the dense V x V matrix of fm_mul for the global A, stored as
 * hmc.c stores it for LAPACK: element (row i, column j) at M[i + j*V].  The
 * couplings are read at every call (hmc.c caches exp(+-mu) at the first). */
void fermion_matrix(_Complex double* M) {
  tg_lattice* L = ctx();
  upload_gauge(A);
  const size_t V = (size_t)NT_ * NX_;
  double* Md = malloc(2 * V * V * sizeof(double));
  if (!Md) {
    fprintf(stderr, "thirring_hmc: fermion_matrix: out of host memory\n");
    exit(1);
  }
  if (tg_dense_M(L, Md) != TG_OK) fatal("tg_dense_M");
  for (size_t i = 0; i < V; i++)
    for (size_t j = 0; j < V; j++) M[i + j * V] = Md[2 * (i * V + j)] + I * Md[2 * (i * V + j) + 1];
  free(Md);
}

/* hmc.c:314-336: det M for the global A.  hmc.c multiplies the diagonal of a
 * LAPACK LU; here the library's GPU LU gives log|det M| and arg det M, and the
 * product is formed once.  As in hmc.c the value overflows a double (inf or
 * NaN parts) once |det M| exceeds 1.8e308 on larger lattices; tg_log_det
 * keeps the logarithm.  V <= 1024. */
double complex determinant(void) {
  tg_lattice* L = ctx();
  upload_gauge(A);
  double logabs = 0, phase = 0;
  if (tg_log_det(L, 1, NULL, &logabs, &phase) != TG_OK) fatal("tg_log_det");
  const double r = exp(logabs);
  return r * cos(phase) + I * (r * sin(phase));
}

/* hmc.c:794-815: 20 stochastic sources, Im c^dag M^dag c averaged. */
double fermion_phase(double*** a) {
  tg_lattice* L = ctx();
  upload_gauge(a);
  int sources = 20;
  double im = 0;
  for (int i = 0; i < sources; i++) {
    for (size_t k = 0; k < (size_t)NT_ * NX_; k++) gauss_pair(&fa[2 * k], &fa[2 * k + 1]);
    if (tg_apply(L, fa, fb, 1) != TG_OK) fatal("tg_apply");
    for (size_t k = 0; k < (size_t)NT_ * NX_; k++) im += fa[2 * k] * fb[2 * k + 1] - fa[2 * k + 1] * fb[2 * k];
  }
  return im / sources;
}

/* hmc.c:823-842 (without the adjoint self-test, whose random vector is still
 * drawn to keep the stream aligned). */
void measure(void) {
  ctx();
  for (size_t k = 0; k < (size_t)NT_ * NX_; k++) {
    double re, im2;
    gauss_pair(&re, &im2);
  }
  double M = 0;
  for (int t = 0; t < NT_; t++)
    for (int x = 0; x < NX_; x++)
      for (int d = 0; d < 2; d++) M += A[t][x][d];
  double phase = fermion_phase(A);
  printf("Magnetisation %g\n", M / (NT_ * NX_));
  printf("Phase %g\n", phase);
}
