/*
 * hmc_main.c -- the `hmc` program of rantahar/Thirring2D (hmc.c:847-943) on
 * the GB300 library: same stdin parameters in the same order
 * (n_loops n_measure m g mu seed), same prompts and output lines, same
 * random stream (seed, 543210 warm-up draws, 100 pure-gauge sweeps from A = 0,
 * then update_gauge / measure).  Lattice size from HMC_NT / HMC_NX (the
 * reference compiles it in; default 32 x 32 as shipped).
 */
#include <stdio.h>
#include <stdlib.h>

#include "thirring_hmc.h"

int main(void) {
  long seed = 0;
  int n_loops = 1, n_measure = 1;

  printf(" Number of updates : ");
  if (scanf("%d", &n_loops) != 1) return 1;
  printf(" Updates / measurement : ");
  if (scanf("%d", &n_measure) != 1) return 1;
  printf(" m : ");
  if (scanf("%lf", &m) != 1) return 1;
  printf(" g : ");
  if (scanf("%lf", &g) != 1) return 1;
  printf(" mu : ");
  if (scanf("%lf", &mu) != 1) return 1;
  printf(" Random number : ");
  if (scanf("%ld", &seed) != 1) return 1;
  seed_mersenne(seed);
  for (int i = 0; i < 543210; i++) (void)mersenne(); /* hmc.c:877 */

  const int nt = thirring_hmc_nt(), nx = thirring_hmc_nx();
  printf(" \n++++++++++++++++++++++++++++++++++++++++++\n");
  printf(" 2D quenched Thirring model, ( %d , %d ) lattice\n", nt, nx);
  printf(" %d updates per measurements\n", n_measure);
  printf(" m %f \n", m);
  printf(" g %f \n", g);
  printf(" mu %f \n", mu);
  printf(" Random seed %ld\n", seed);

  /* fields with the reference's shapes: NX+1 columns (hmc.c:888-898) */
  eta = malloc(nt * sizeof(int**));
  A = malloc(nt * sizeof(double**));
  for (int t = 0; t < nt; t++) {
    A[t] = malloc((nx + 1) * sizeof(double*));
    eta[t] = malloc((nx + 1) * sizeof(int*));
    for (int x = 0; x < nx + 1; x++) {
      eta[t][x] = calloc(2, sizeof(int));
      A[t][x] = calloc(2, sizeof(double));
    }
  }
  xup = malloc((nx + 1) * sizeof(int));
  xdn = malloc((nx + 1) * sizeof(int));
  tup = malloc(nt * sizeof(int));
  tdn = malloc(nt * sizeof(int));
  for (int i = 0; i < nt; i++) { tup[i] = (i + 1) % nt; tdn[i] = (i - 1 + nt) % nt; }
  for (int i = 0; i < nx + 1; i++) { xup[i] = (i + 1) % nx; xdn[i] = (i - 1 + nx) % nx; }
  for (int t = 0; t < nt; t++)
    for (int x = 0; x < nx; x++) {
      eta[t][x][1] = 1;
      eta[t][x][0] = (x % 2 == 0) ? 1 : -1;
    }

  for (int i = 0; i < 100; i++) update_puregauge_hb(A); /* hmc.c:927-929 */

  for (int i = 1; i < n_loops + 1; i++) {
    update_gauge(A);
    if ((i % n_measure) == 0) measure();
    fflush(stdout);
  }
  return 0;
}
