/*
 * ref_driver.c -- in-process driver for the generated, adjoint-corrected copy
 * of the reference hmc.c (built by oracle/make_ref.py into oracle/_ref/).
 *
 * TEST INFRASTRUCTURE ONLY: it lets the parity tests and the CPU reference
 * arm of bench.py call the reference's own functions on flat arrays.  It
 * #includes the generated source, so NT, NX, the globals (m, g, mu, A, eta,
 * tup/tdn/xup/xdn) and every function of hmc.c are in scope.
 *
 * Flat layouts: A and momenta double[NT*NX*2] ([t][x][dir]); fermion vectors
 * complex double[NT*NX] ([t][x]), passed as interleaved doubles.
 */
#include "hmc_patched.c"

void LAPACK_zgetrf(int* m_, int* n_, _Complex double* a_, int* lda_, int* ipiv_, int* info_) {
  (void)m_; (void)n_; (void)a_; (void)lda_; (void)ipiv_; (void)info_;
  fprintf(stderr, "ref_driver: LAPACK is not available in the oracle build\n");
  abort();
}

static _Complex double** vin;
static _Complex double** vout;
static double*** momv;

int ref_nt(void) { return NT; }
int ref_nx(void) { return NX; }

/* Lattice set-up equivalent to hmc.c:874-925 without stdin: parameters,
 * seeded RNG with `warmup` discarded draws (hmc.c:877 uses 543210), A = 0,
 * neighbour tables and staggered phases. */
void ref_setup(double m_, double g_, double mu_, long seed, int warmup) {
  m = m_;
  g = g_;
  mu = mu_;
  seed_mersenne(seed);
  for (int i = 0; i < warmup; i++) mersenne();
  eta = malloc(NT * sizeof(int**));
  A = malloc(NT * sizeof(double**));
  momv = malloc(NT * sizeof(double**));
  for (int t = 0; t < NT; t++) {
    A[t] = malloc((NX + 1) * sizeof(double*));
    eta[t] = malloc((NX + 1) * sizeof(int*));
    momv[t] = malloc(NX * sizeof(double*));
    for (int x = 0; x < NX + 1; x++) {
      eta[t][x] = malloc(ND * sizeof(int));
      A[t][x] = malloc(ND * sizeof(double));
      A[t][x][0] = A[t][x][1] = 0;
      eta[t][x][0] = eta[t][x][1] = 0;
      if (x < NX) momv[t][x] = malloc(ND * sizeof(double));
    }
  }
  xup = malloc((NX + 1) * sizeof(int));
  xdn = malloc((NX + 1) * sizeof(int));
  tup = malloc(NT * sizeof(int));
  tdn = malloc(NT * sizeof(int));
  for (int i = 0; i < NT; i++) { tup[i] = (i + 1) % NT; tdn[i] = (i - 1 + NT) % NT; }
  for (int i = 0; i < NX + 1; i++) { xup[i] = (i + 1) % NX; xdn[i] = (i - 1 + NX) % NX; }
  for (int t = 0; t < NT; t++)
    for (int x = 0; x < NX; x++) {
      eta[t][x][1] = 1;
      eta[t][x][0] = (x % 2 == 0) ? 1 : -1;
    }
  vin = alloc_vector();
  vout = alloc_vector();
}

void ref_set_A(const double* a) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++)
    A[t][x][d] = a[(t * NX + x) * ND + d];
}
void ref_get_A(double* a) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++)
    a[(t * NX + x) * ND + d] = A[t][x][d];
}

static void to_rows(const double* f, _Complex double** v) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) {
    int s = t * NX + x;
    v[t][x] = f[2 * s] + I * f[2 * s + 1];
  }
}
static void from_rows(_Complex double** v, double* f) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) {
    int s = t * NX + x;
    f[2 * s] = creal(v[t][x]);
    f[2 * s + 1] = cimag(v[t][x]);
  }
}
static void mom_in(const double* f) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++)
    momv[t][x][d] = f[(t * NX + x) * ND + d];
}
static void mom_out(double* f) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++)
    f[(t * NX + x) * ND + d] = momv[t][x][d];
}

double ref_mersenne(void) { return mersenne(); }
void ref_mersenne_fill(double* out, long n) { for (long k = 0; k < n; k++) out[k] = mersenne(); }

void ref_puregauge(int sweeps) { for (int i = 0; i < sweeps; i++) update_puregauge_hb(A); }

void ref_fm_mul(const double* in, double* out) { to_rows(in, vin); fm_mul(vin, vout, A); from_rows(vout, out); }
void ref_fm_conjugate_mul(const double* in, double* out) {
  to_rows(in, vin); fm_conjugate_mul(vin, vout, A); from_rows(vout, out);
}
/* fmdm_invert_cg, hmc.c:341-404 (exits the process on divergence) */
void ref_cg(const double* b, double* x) { to_rows(b, vin); fmdm_invert_cg(vin, vout, A); from_rows(vout, x); }

double ref_gauge_action(void) { return calc_gauge_action(A); }
double ref_pseudofermion_action(const double* phi) { to_rows(phi, vin); return pseudofermion_action(vin, A); }
double ref_md_action(const double* n) { to_rows(n, vin); return stochastic_md_action(vin, A); }

/* random_pseudofermion (hmc.c:418-436): draws V pairs, writes phi, returns sum|eta|^2 */
double ref_random_pseudofermion(double* phi) {
  double s = random_pseudofermion(vout, A);
  from_rows(vout, phi);
  return s;
}
double ref_random_momentum(double* p) { double s = random_momentum(momv); mom_out(p); return s; }
void ref_stochastic_vector(double* n) { stochastic_vector(vout); from_rows(vout, n); }

/* momentum_step (hmc.c:504-665) on p, using the current A */
void ref_momentum_step(double* p, const double* psi, const double* st, double eps) {
  _Complex double** ps = alloc_vector();
  _Complex double** sv = alloc_vector();
  to_rows(psi, ps);
  to_rows(st, sv);
  mom_in(p);
  momentum_step(momv, A, ps, sv, eps);
  mom_out(p);
  free_vector(ps);
  free_vector(sv);
}
void ref_gauge_step(const double* p, double eps) { mom_in(p); gauge_step(A, momv, eps); }

/* The reference's own update_gauge (hmc.c:671-746: 10 leapfrog steps of a
 * trajectory of length 1, its CG stopping at |r|^2 < 1e-30), called as the
 * main loop of hmc.c:932-939 calls it.  It prints its action lines and the
 * decision to stdout.  Used to time whole reference trajectories. */
void ref_update_gauge(void) { update_gauge(A); }

/* One trajectory with the sequence of update_gauge (hmc.c:671-746) built from
 * the reference's own functions, with nsteps/tau as arguments (the reference
 * hard-codes 10 and 1) and the stats returned at full precision instead of
 * printed with %g.  stats = dH, Sg0, Spf0, Smd0, Smom0, Sg1, Spf1, Smd1, Smom1,
 * accepted. */
void ref_trajectory(int nsteps, double tau, double* stats) {
  _Complex double** psi = alloc_vector();
  _Complex double** chi = alloc_vector();
  double*** newA = malloc(NT * sizeof(double**));
  for (int t = 0; t < NT; t++) {
    newA[t] = malloc((NX + 1) * sizeof(double*));
    for (int x = 0; x < NX + 1; x++) newA[t][x] = calloc(ND, sizeof(double));
  }
  double Spf0 = random_pseudofermion(psi, A);
  double Smom0 = random_momentum(momv);
  double Sg0 = calc_gauge_action(A);
  stochastic_vector(chi);
  double Smd0 = stochastic_md_action(chi, A);
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++) newA[t][x][d] = A[t][x][d];
  for (int i = 0; i < nsteps; i++) {
    gauge_step(newA, momv, tau * 0.5 / nsteps);
    momentum_step(momv, newA, psi, chi, tau / nsteps);
    gauge_step(newA, momv, tau * 0.5 / nsteps);
  }
  double Spf1 = pseudofermion_action(psi, newA);
  double Smom1 = 0;
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++)
    Smom1 += momv[t][x][d] * momv[t][x][d];
  double Sg1 = calc_gauge_action(newA);
  double Smd1 = stochastic_md_action(chi, newA);
  double dS = Smom1 - Smom0 + Spf1 - Spf0 + Smd1 - Smd0 + Sg1 - Sg0;
  int acc = exp(-dS) > mersenne();
  if (acc)
    for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) for (int d = 0; d < ND; d++) A[t][x][d] = newA[t][x][d];
  double out[10] = {dS, Sg0, Spf0, Smd0, Smom0, Sg1, Spf1, Smd1, Smom1, (double)acc};
  for (int k = 0; k < 10; k++) stats[k] = out[k];
  for (int t = 0; t < NT; t++) { for (int x = 0; x < NX + 1; x++) free(newA[t][x]); free(newA[t]); }
  free(newA);
  free_vector(psi);
  free_vector(chi);
}

/* fermion_matrix (hmc.c:269-310): the dense V x V matrix, stored as the
 * reference stores it (element (row i, column j) at M[i + j*V]). */
void ref_fermion_matrix(double* out) {
  _Complex double* M = malloc((size_t)VOLUME * VOLUME * sizeof(_Complex double));
  fermion_matrix(M);
  for (long k = 0; k < (long)VOLUME * VOLUME; k++) { out[2 * k] = creal(M[k]); out[2 * k + 1] = cimag(M[k]); }
  free(M);
}
