/*
 * vecops_driver.c -- in-process driver for the reference's own vec_ops.c (the
 * fermion-bag programs' masked real operator and CG), compiled by
 * oracle/make_ref.py against a copy of Thirring.h whose NT/NX come from -D.
 *
 * TEST INFRASTRUCTURE ONLY.  Defines the globals Thirring.h declares (MAIN),
 * sets up the lattice as fermionbag.c:696-775 does (neighbour tables wrapping
 * mod NT/NX, eta_t = (-1)^x, eta_x = 1, all sites empty) and exposes flat
 * arrays: fields double[NT*NX] t-major, occupation int[NT*NX].
 */
#define MAIN
#include "Thirring.h"

void LAPACK_zgetrf(int* m_, int* n_, _Complex double* a_, int* lda_, int* ipiv_, int* info_) {
  (void)m_; (void)n_; (void)a_; (void)lda_; (void)ipiv_; (void)info_;
  abort();
}

static double **vin, **vout;

int vref_nt(void) { return NT; }
int vref_nx(void) { return NX; }

void vref_setup(double m_, double mu_) {
  m = m_;
  mu = mu_;
  field = malloc(NT * sizeof(int*));
  eta = malloc(NT * sizeof(int**));
  for (int t = 0; t < NT; t++) {
    field[t] = calloc(NX + 1, sizeof(int));
    eta[t] = malloc((NX + 1) * sizeof(int*));
    for (int x = 0; x < NX + 1; x++) {
      eta[t][x] = malloc(2 * sizeof(int));
      eta[t][x][0] = (x % 2 == 0) ? 1 : -1;
      eta[t][x][1] = 1;
    }
  }
  xup = malloc((NX + 1) * sizeof(int));
  xdn = malloc((NX + 1) * sizeof(int));
  tup = malloc(NT * sizeof(int));
  tdn = malloc(NT * sizeof(int));
  for (int i = 0; i < NT; i++) { tup[i] = (i + 1) % NT; tdn[i] = (i - 1 + NT) % NT; }
  for (int i = 0; i < NX + 1; i++) { xup[i] = (i + 1) % NX; xdn[i] = (i - 1 + NX) % NX; }
  vin = alloc_vector();
  vout = alloc_vector();
}

void vref_set_field(const int* f) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) field[t][x] = f[t * NX + x];
}

static void to_rows(const double* f, double** v) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) v[t][x] = f[t * NX + x];
}
static void from_rows(double** v, double* f) {
  for (int t = 0; t < NT; t++) for (int x = 0; x < NX; x++) f[t * NX + x] = v[t][x];
}

/* fM(chi, psi) / fM_transpose(chi, psi): chi = output (vec_ops.c:96, 135) */
void vref_fM(const double* in, double* out, int transpose) {
  to_rows(in, vin);
  if (transpose) fM_transpose(vout, vin);
  else fM(vout, vin);
  from_rows(vout, out);
}

/* cg_MdM(inv, source), vec_ops.c:261 */
void vref_cg_MdM(const double* b, double* x) {
  to_rows(b, vin);
  cg_MdM(vout, vin);
  from_rows(vout, x);
}

#ifdef PROPAGATOR_MATRIX
/* calc_Dinv (fermion_matrix.c:189-351, built with PROPAGATOR_MATRIX and
 * WITH_MASS_MONOMERS) for the current field; out: double[NT*NX*NT*NX/2] in the
 * reference's layout.  calc_Dinv reads a cached propagator file from the
 * working directory if one exists and writes one: call it from an empty
 * directory. */
double* Dinv;

void vref_calc_Dinv(double* out) {
  const size_t n = (size_t)NT * NX * NT * NX / 2;
  Dinv = malloc(n * sizeof(double));
  calc_Dinv();
  for (size_t i = 0; i < n; i++) out[i] = Dinv[i];
  free(Dinv);
  Dinv = NULL;
}
#endif
