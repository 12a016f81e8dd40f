/*
 * det_driver.c -- in-process driver for the reference's full_determinant.c
 * (determinant_mu, full_determinant.c:144-186) built with fermion_matrix.c's
 * fM_index (fermion_matrix.c:28-186) by oracle/make_ref.py into oracle/_ref/.
 *
 * TEST INFRASTRUCTURE ONLY: it produces the determinant goldens that pin the
 * library's dense operator and log-determinant on tiny lattices.
 *
 * The generated Thirring.h fixes NT and NX (REF_NT, REF_NX), the boundary
 * (antisymmetric in both directions, or with REF_OPENX open in x and
 * antisymmetric in t) and leaves FLUCTUATION_MATRIX undefined, which is what
 * compiles determinant_mu.  Without WITH_MASS_MONOMERS the mass m sits on
 * fM_index's diagonal, so with no occupied site determinant_mu is det(m + D).
 * Set-up as the fermion-bag programs do it (fermionbag.c:713-790): neighbour
 * tables, the open-x phantom column NX, staggered phases eta_t = (-1)^x,
 * eta_x = 1, an empty field.
 */
#define MAIN
#include "Thirring.h"

double* Dinv;
int *evenlist, *oddlist;
int current_sign;

double determinant_mu(double mu_);

void dref_setup(double m_, double mu_) {
  m = m_;
  mu = mu_;
  U = 0;
  n_monomers = n_links = 0;
  field = malloc(NT * sizeof(int*));
  eta = malloc(NT * sizeof(int**));
  for (int t = 0; t < NT; t++) {
    field[t] = malloc((NX + 1) * sizeof(int));
    eta[t] = malloc((NX + 1) * sizeof(int*));
    for (int x = 0; x < NX + 1; x++) {
      eta[t][x] = malloc(2 * sizeof(int));
      eta[t][x][0] = eta[t][x][1] = 0;
      field[t][x] = 0;
    }
  }
  xup = malloc((NX + 1) * sizeof(int));
  xdn = malloc((NX + 1) * sizeof(int));
  tup = malloc(NT * sizeof(int));
  tdn = malloc(NT * sizeof(int));
  for (int i = 0; i < NT; i++) {
    tup[i] = (i + 1) % NT;
    tdn[i] = (i - 1 + NT) % NT;
  }
  for (int i = 0; i < NX + 1; i++) {
    xup[i] = (i + 1) % NX;
    xdn[i] = (i - 1 + NX) % NX;
  }
#ifdef OPENX
  xdn[0] = NX;
  xup[NX - 1] = NX;
  xup[NX] = NX;
  for (int t = 0; t < NT; t++) field[t][NX] = EMPTY;
#endif
  for (int t = 0; t < NT; t++)
    for (int x = 0; x < NX; x++) {
      eta[t][x][1] = 1;
      eta[t][x][0] = (x % 2 == 0) ? 1 : -1;
    }
}

/* mask[t*NX + x] != 0: the site is occupied (a monomer) and leaves the matrix */
void dref_set_field(const int* mask) {
  n_monomers = 0;
  for (int t = 0; t < NT; t++)
    for (int x = 0; x < NX; x++) {
      field[t][x] = mask[t * NX + x] ? MONOMER : 0;
      n_monomers += mask[t * NX + x] ? 1 : 0;
    }
}

double dref_determinant_mu(double mu_) { return determinant_mu(mu_); }
