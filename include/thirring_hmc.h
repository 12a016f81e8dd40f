/*
 * thirring_hmc.h -- drop-in for the function set of rantahar/Thirring2D hmc.c
 * (and mersenne.h), implemented on the GB300 library (include/thirring_gpu.h).
 *
 * A program written against hmc.c's functions links libthirring_hmc.so
 * instead of hmc.o + mersenne_inline.o: same names, same argument orders,
 * same row-pointer array layouts, same globals, same random-number stream and
 * the same printed lines.  The work runs on the GPU; the layer gathers the
 * caller's row-pointer arrays into contiguous buffers and back.
 *
 * Differences, all deliberate:
 *  - NT and NX are run-time values (hmc.c:14-15 fixes them at compile time):
 *    thirring_hmc_set_lattice(), or the environment HMC_NT / HMC_NX, default 32
 *    x 32 as hmc.c ships.
 *  - fm_conjugate_mul applies the true adjoint of fm_mul.  hmc.c:188-249 ships
 *    a verbatim copy of fm_mul, with which its CG diverges on every lattice.
 *  - x boundary: antiperiodic as hmc.c:165-180 ships, or periodic with
 *    HMC_BC_X=periodic.
 *  - CG: hmc.c's stop |r|^2 < 1e-30 and cap 100000 by default; HMC_CG_REL=<tol>
 *    switches to a relative stop and HMC_PRECISION=mixed to the FP32 solver
 *    with FP64 reliable updates.
 *  - measure() skips the self-test test_conjugate (hmc.c:759-789), which checks
 *    an identity that a correct adjoint does not satisfy, but still draws its
 *    random vector so the stream stays aligned with hmc.c.
 *  - Failures print hmc.c's message and exit(1) as hmc.c does
 *    (hmc.c:383-386); CUDA errors print the CUDA message and exit(1).
 */
#ifndef THIRRING_HMC_H
#define THIRRING_HMC_H

#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- globals of hmc.c:38-50 ------------------------------------------- */
extern double m;
extern double g;
extern double mu;
extern int *tup, *xup, *tdn, *xdn;
extern double*** A;
extern int*** eta;

/* ---- random numbers: mersenne.h / mersenne_inline.c ------------------- */
#define MERSENNE_N 624
extern int mersenne_i;
extern double mersenne_array[MERSENNE_N];
#define mersenne() (mersenne_i > 0 ? mersenne_array[--mersenne_i] : mersenne_generate())
void seed_mersenne(long seed);       /* mersenne_inline.c:73-87  */
double mersenne_generate(void);      /* mersenne_inline.c:89-128 */

/* ---- lattice size (compile-time NT/NX in hmc.c:14-15) ------------------ */
void thirring_hmc_set_lattice(int nt, int nx);
int thirring_hmc_nt(void);
int thirring_hmc_nx(void);

/* ---- hmc.c entry points ------------------------------------------------ */
_Complex double** alloc_vector(void);                                                    /* hmc.c:105 */
void free_vector(_Complex double** v);                                                   /* hmc.c:115 */
void fm_mul(_Complex double** v_in, _Complex double** v_out, double*** A);               /* hmc.c:123 */
void fm_conjugate_mul(_Complex double** v_in, _Complex double** v_out, double*** A);     /* hmc.c:188 */
void fmdm_invert_cg(_Complex double** v_in, _Complex double** v_out, double*** A);       /* hmc.c:341 */
void fm_invert_cg(_Complex double** v_in, _Complex double** v_out, double*** A);         /* hmc.c:408 */
double random_pseudofermion(_Complex double** v, double*** A);                           /* hmc.c:418 */
void stochastic_vector(_Complex double** v);                                             /* hmc.c:439 */
double pseudofermion_action(_Complex double** v, double*** A);                           /* hmc.c:451 */
double stochastic_md_action(_Complex double** v, double*** A);                           /* hmc.c:467 */
double random_momentum(double*** mom);                                                   /* hmc.c:483 */
double momentum_step(double*** mom, double*** A, _Complex double** psi, _Complex double** st,
                     double eps);                                                        /* hmc.c:504 */
double gauge_step(double*** A, double*** mom, double eps);                               /* hmc.c:97  */
double calc_gauge_action(double*** A);                                                   /* hmc.c:73  */
void update_puregauge_hb(double*** A);                                                   /* hmc.c:82  */
void update_gauge(double*** A);                                                          /* hmc.c:671 */
void fermion_matrix(_Complex double* M);  /* hmc.c:269: M[i + j*V], global A; V <= 4096 */
_Complex double determinant(void);        /* hmc.c:314: global A; V <= 1024; overflows as hmc.c's */
double fermion_phase(double*** A);                                                       /* hmc.c:794 */
void measure(void);                                                                      /* hmc.c:823 */

#ifdef __cplusplus
}
#endif
#endif /* THIRRING_HMC_H */
