/*
 * thirring_gpu.h -- C ABI of the GB300 (sm_103a) Thirring2D HMC library.
 *
 * One tg_lattice holds one lattice (NT x NX sites), its couplings, its
 * device-resident fields and a CUDA stream.  All entry points take plain
 * pointers and sizes; "host" buffers are ordinary CPU memory, "_dev" buffers
 * are device pointers on the lattice's device.  Every call returns a status
 * (TG_OK = 0); tg_last_error() gives the message of the last failure on the
 * calling thread.  Nothing here calls exit().  Calls that run CG return the
 * solver's status (TG_E_NOCONV, TG_E_DIVERGED, TG_E_NAN) when a solve did not
 * converge; their outputs and result structs are still written.
 *
 * Field layouts (identical to the reference's row-pointer arrays flattened
 * t-major, hmc.c:105-112 and 888-898):
 *   gauge field / momenta / forces   double[NT*NX*2]   index (t*NX + x)*2 + dir
 *   fermion vectors                  double[NT*NX*2]   interleaved (re, im) of
 *                                                      complex v[t][x]
 *
 * The reference (rantahar/Thirring2D) has no library; its interface is the
 * function set of hmc.c.  Each entry point below names the function it
 * replaces.  include/thirring_hmc.h declares the drop-in with the
 * reference's exact names and signatures, built on top of this API.
 */
#ifndef THIRRING_GPU_H
#define THIRRING_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TG_OK 0
#define TG_E_NOCONV 1   /* CG reached maxiter (hmc.c:364 stops silently)                      */
#define TG_E_DIVERGED 2 /* |r|^2/|r0|^2 > 1e10 (hmc.c:383-386: "Cannot invert fermion matrix") */
#define TG_E_NAN 3      /* NaN in a CG recurrence                                             */
#define TG_E_CUDA 4     /* CUDA runtime error                                                 */
#define TG_E_ARG 5      /* invalid argument                                                   */
#define TG_E_ALLOC 6    /* device or pinned allocation failed                                 */
#define TG_E_TIMEOUT 7  /* a grid barrier of the persistent solver waited past its limit      */

/* ---- boundary conditions (sign of the hop across the last slice) ------- */
#define TG_BC_PERIODIC 1
#define TG_BC_ANTIPERIODIC (-1) /* hmc.c:143-148 (t) and 165-180 (x) as shipped */
#define TG_BC_OPEN 0

/* ---- solver precision --------------------------------------------------- */
#define TG_PREC_FP64 0  /* all of CG in FP64, the reference's arithmetic          */
#define TG_PREC_MIXED 1 /* FP32 CG with FP64 reliable updates of x and b - A x    */

/* ---- random numbers of a trajectory --------------------------------------- */
#define TG_RNG_MT 0       /* the reference's MT19937 stream (mersenne.h), drawn on the host */
#define TG_RNG_PHILOX 1   /* Philox4x32-10 on the device, keyed by seed and trajectory      */
#define TG_RNG_EXTERNAL 2 /* caller supplies the Gaussian fields (tg_trajectory_ext)        */

typedef struct tg_lattice tg_lattice;

typedef struct {
  int nt, nx;       /* NT, NX (hmc.c:14-15, compile-time constants there)  */
  double m, g, mu;  /* mass, coupling, chemical potential (hmc.c:38-40)    */
  int bc_t, bc_x;   /* TG_BC_*; the reference ships ANTIPERIODIC for both  */
  int device;       /* CUDA device ordinal                                  */
} tg_lattice_params;

typedef struct {
  double rel_tol;   /* stop when |r| < rel_tol |b| (0 disables)                      */
  double abs_tol2;  /* stop when |r|^2 < abs_tol2 (hmc.c:34 CG_ACCURACY = 1e-30)     */
  int maxiter;      /* iteration cap (hmc.c:35 CG_MAX_ITER = 100000)                  */
  int precision;    /* TG_PREC_*                                                      */
  int ru_interval;  /* TG_PREC_MIXED: FP32 iterations between FP64 reliable updates   */
  int solver;       /* TG_SOLVER_*: how the iterations are scheduled (0 = default)    */
} tg_cg_params;

/* tg_cg_params.solver.  Both run the same iteration and stopping rules; they
 * differ in rounding of the grid sums only. */
#define TG_SOLVER_DEFAULT 0     /* the faster of the two on this library's measurements:
                                   persistent (TG_SOLVER=launches|persistent overrides)    */
#define TG_SOLVER_LAUNCHES 1    /* two kernel launches per iteration (graph WHILE node)       */
#define TG_SOLVER_PERSISTENT 2  /* one cooperative launch per solve, grid barriers inside     */

typedef struct {
  int iterations;       /* CG iterations (each = one M and one M^dagger apply) */
  int status;           /* TG_OK, TG_E_NOCONV, TG_E_DIVERGED or TG_E_NAN        */
  int reliable_updates; /* TG_PREC_MIXED only                                   */
  int pad_;
  double rr;            /* final |r|^2 (true residual after a reliable update)  */
  double rr0;           /* |b|^2                                                */
} tg_cg_result;

typedef struct {
  int nsteps;              /* leapfrog steps (hmc.c:708 uses 10)                          */
  double tau;              /* trajectory length (hmc.c:709 uses 1)                         */
  int npf;                 /* pseudofermions (hmc.c uses 1; at most 8)                     */
  int stochastic_term;     /* 1: include Re <n, M^dag n> and its force (hmc.c:467-479,
                              608-661, 698-699) -- it consumes V Gaussian pairs per
                              trajectory and vanishes identically at mu = 0              */
  int rng;                 /* TG_RNG_MT or TG_RNG_PHILOX for tg_trajectory                 */
  int use_graph;           /* 1: run the trajectory as one CUDA graph (a persistent
                              solve is one node; launch-per-iteration CG loops are
                              conditional WHILE nodes); 0: eager launches              */
  unsigned long long seed; /* Philox key                                                  */
  tg_cg_params cg;         /* solver used inside the trajectory                           */
} tg_hmc_params;

typedef struct {
  double dH;                         /* H_end - H_start, hmc.c:729-732 order  */
  double Sg0, Spf0, Smd0, Smom0;     /* actions at the start (hmc.c:695-699)  */
  double Sg1, Spf1, Smd1, Smom1;     /* actions at the end (hmc.c:719-726)    */
  double u_accept;                   /* the uniform compared with exp(-dH)    */
  int accepted;                      /* exp(-dH) > u  (hmc.c:738)             */
  int status;                        /* worst CG status of the trajectory     */
  int cg_solves, cg_iterations;      /* totals over the trajectory            */
  int cg_max_iterations, reliable_updates;
  double cg_ms;                      /* device time inside CG solves          */
} tg_traj_result;

/* ---- context ------------------------------------------------------------ */
const char* tg_last_error(void);
const char* tg_version(void);
/* Allocates every device field of the lattice (about 40 x 16 B x NT*NX).
 * A starts at 0, as hmc.c:896. */
int tg_create(const tg_lattice_params* p, tg_lattice** out);
int tg_destroy(tg_lattice* L);
/* m, g, mu are globals the reference reads at every call (hmc.c:38-40). */
int tg_set_couplings(tg_lattice* L, double m, double g, double mu);
int tg_get_params(const tg_lattice* L, tg_lattice_params* p);
int tg_synchronize(tg_lattice* L);
void* tg_stream(tg_lattice* L); /* the lattice's cudaStream_t */

/* ---- gauge field: the reference's global double ***A (hmc.c:47) --------- */
int tg_set_gauge(tg_lattice* L, const double* A);
int tg_get_gauge(tg_lattice* L, double* A);
int tg_set_gauge_dev(tg_lattice* L, const void* A_dev);

/* ---- operator ---------------------------------------------------------- */
/* fm_mul (hmc.c:123-184): out = M in.  dagger = 1: fm_conjugate_mul
 * (hmc.c:188-249) as the true adjoint M^dagger = m - D(-mu).  The shipped
 * fm_conjugate_mul is a verbatim copy of fm_mul, which makes the reference's
 * CG diverge; this library applies the adjoint.  Host buffers, FP64. */
int tg_apply(tg_lattice* L, const double* in, double* out, int dagger);
/* Same on device vectors: double2[V] for TG_PREC_FP64, float2[V] for
 * TG_PREC_MIXED (the FP32 operator).  Enqueued on the lattice's stream. */
int tg_apply_dev(tg_lattice* L, const void* in, void* out, int dagger, int precision);
/* Times n back-to-back applies on device vectors with CUDA events on the
 * lattice's stream; *ms_per_apply = average per launch. */
int tg_time_apply(tg_lattice* L, int n, int dagger, int precision, double* ms_per_apply);

/* ---- CG on M^dagger M: fmdm_invert_cg (hmc.c:341-404) -------------------- */
int tg_cg(tg_lattice* L, const tg_cg_params* cp, const double* b, double* x, tg_cg_result* res);
int tg_cg_dev(tg_lattice* L, const tg_cg_params* cp, const void* b_dev, void* x_dev, tg_cg_result* res);

/* ---- actions and forces ------------------------------------------------- */
/* calc_gauge_action (hmc.c:73-79) of the lattice's gauge field. */
int tg_gauge_action(tg_lattice* L, double* S);
/* pseudofermion_action (hmc.c:451-463): Re <phi, (M^dag M)^-1 phi>. */
int tg_pseudofermion_action(tg_lattice* L, const tg_cg_params* cp, const double* phi, double* S,
                            tg_cg_result* res);
/* stochastic_md_action (hmc.c:467-479): Re <n, M^dag n>. */
int tg_md_action(tg_lattice* L, const double* n, double* S);
/* dS/dA on every link (gauge + pseudofermion + stochastic term), the force
 * momentum_step (hmc.c:504-661) subtracts, from npf solved vectors
 * chi_k = (M^dag M)^-1 phi_k (double[npf*V*2]); noise may be NULL. */
int tg_force(tg_lattice* L, int npf, const double* chi, const double* noise, double* F);
/* dS_pf/dA alone -- the pseudofermion force of hmc.c:517-576, summed over
 * npf pseudofermions phi (double[npf*V*2]) -- solving chi_k = (M^dag M)^-1
 * phi_k afresh (the solution is not kept).  F: double[V*2]. */
int tg_pf_force(tg_lattice* L, const tg_cg_params* cp, int npf, const double* phi, double* F, tg_cg_result* res);
/* momentum_step (hmc.c:504-665): mom -= eps * dS/dA, solving for every
 * pseudofermion; res (may be NULL) receives the summed CG counts. */
int tg_momentum_step(tg_lattice* L, const tg_cg_params* cp, double* mom, int npf, const double* phi,
                     const double* noise, double eps, tg_cg_result* res);
/* gauge_step (hmc.c:97-101): A += 2 eps mom. */
int tg_gauge_step(tg_lattice* L, const double* mom, double eps);

/* ---- random numbers: the reference stream (mersenne_inline.c) ------------ */
/* seed_mersenne(seed) then `warmup` discarded draws (hmc.c:874-877 uses 543210). */
int tg_mt_seed(tg_lattice* L, long seed, long warmup);
int tg_mt_uniforms(tg_lattice* L, double* out, long n);
/* update_puregauge_hb (hmc.c:82-93) x sweeps, drawing from the MT stream.
 * Links are independent, so each sweep is one data-parallel kernel. */
int tg_puregauge_sweeps(tg_lattice* L, int sweeps);
/* Same with caller-supplied uniforms: u[sweeps * 4 * NT*NX], per link (t-major,
 * dir inner) the proposal uniform then the acceptance uniform. */
int tg_puregauge_ext(tg_lattice* L, const double* u, int sweeps);

/* ---- checkpoint and resume ------------------------------------------------
 * hmc.c keeps no state between runs (fermionbag.c:125-163 writes its raw
 * field).  A checkpoint holds everything a resumed run needs to continue
 * bitwise: couplings, the reference MT stream (words and pending outputs),
 * the Philox trajectory counter and A.  Little-endian layout, byte offsets:
 *   0  char[8] "TGCKPT01"      8  int32 version (1)     12 int32 nt
 *   16 int32 nx                20 int32 bc_t            24 int32 bc_x
 *   28 int32 MT outputs left   32 int32 MT seeded       36 int32 (0)
 *   40 double m                48 double g              56 double mu
 *   64 uint64 Philox trajectory counter
 *   72 uint32[624] MT words    2568 double[624] MT outputs of the current block
 *   7560 double[nt*nx*2] A ([t][x][dir], as tg_set_gauge).
 * Loading needs a lattice of the same nt, nx and boundary conditions. */
size_t tg_checkpoint_size(const tg_lattice* L);
int tg_checkpoint_save(tg_lattice* L, void* buf, size_t size);
int tg_checkpoint_load(tg_lattice* L, const void* buf, size_t size);

/* ---- HMC trajectory: update_gauge (hmc.c:671-746) ------------------------- */
/* Draws the pseudofermion, momentum, noise fields and the accept uniform
 * from the stream p->rng selects (TG_RNG_MT: the reference's order, so the
 * trajectory reproduces hmc.c's on the same seed), runs the leapfrog on the
 * device, accepts or rejects, and leaves the new A on the device. */
int tg_trajectory(tg_lattice* L, const tg_hmc_params* p, tg_traj_result* r);
/* Same with caller-supplied fields: eta double[npf*V*2] (phi_k = M^dag eta_k),
 * mom double[V*2], noise double[V*2] (ignored unless stochastic_term),
 * u_accept the uniform of hmc.c:738. */
int tg_trajectory_ext(tg_lattice* L, const tg_hmc_params* p, const double* eta, const double* mom,
                      const double* noise, double u_accept, tg_traj_result* r);

/* ---- measurements -------------------------------------------------------- */
/* magnetisation of measure() (hmc.c:831-839): sum of A over sites and
 * directions divided by NT*NX. */
int tg_magnetisation(tg_lattice* L, double* M);
/* fermion_phase (hmc.c:794-815): (1/sources) sum_k Im <c_k, M^dag c_k> over
 * Gaussian sources.  noise: double[sources*V*2], or NULL to draw V pairs per
 * source from the lattice's reference MT stream in hmc.c's order. */
int tg_fermion_phase(tg_lattice* L, int sources, const double* noise, double* phase);
/* Stochastic chiral condensate (no counterpart in hmc.c):
 * pbp = (1/2V) mean_k Re <eta_k, M^-1 eta_k> over `sources` complex Gaussian
 * Philox sources (E[eta eta^dag] = 2), M^-1 = (M^dag M)^-1 M^dag by CG;
 * *err = standard error over the sources (may be NULL). */
int tg_chiral_condensate(tg_lattice* L, const tg_cg_params* cp, int sources, unsigned long long seed, double* pbp,
                         double* err);

/* ---- measurement utility (no reference counterpart) ---------------------- */
/* FP64 FMA throughput of `device` in TFLOP/s (2 flops per FMA; the best of
 * timed launches of a kernel of independent FMA chains at 2, 4 and 8 blocks of
 * 256 threads per SM, CUDA events).  The
 * FP64 roof against which the FP64 operator and CG kernels are reported. */
int tg_measure_fp64_peak(int device, double* tflops);
/* Waits of the shared-memory-staged FP32 stencil kernels that gave up (their
 * bounded wait on a TMA copy ran out) since the library was loaded: 0 in a
 * healthy run.  No reference counterpart. */
int tg_stage_faults(int device, unsigned* count);
/* The persistent solver's grid barrier on its failure path: one barrier on a
 * small cooperative grid that also waits for phantom_blocks blocks that do not
 * exist.  *status = TG_OK when it was passed (phantom_blocks = 0), TG_E_TIMEOUT
 * when it gave up after its bounded wait (tens of milliseconds); the device
 * stays usable either way.  No reference counterpart. */
int tg_grid_barrier_check(int device, int phantom_blocks, int* status);

/* ---- fermion-bag propagator matrix ----------------------------------------- */
/* calc_Dinv with WITH_MASS_MONOMERS (fermion_matrix.c:189-351): for every
 * source site the column fM^-1 e_src of the masked real operator, each by
 * cg_propagator (vec_ops.c:311-321, CG on fM^T fM with b = fM^T e_src, the
 * stopping rules of cp; the reference uses abs_tol2 = 1e-30 and 9999
 * iterations).  mask: occupation int[V] as for tg_fm_apply, or NULL for the
 * free propagator.  Dinv: double[V*V/2] laid out as the reference's Dinv
 * (n = V/2, i = (nx*t + x)/2): Dinv[i2*n + i1] for odd sources i1 and even
 * sites i2, Dinv[n*n + i2*n + i1] for even sources and odd sites.  A source
 * whose CG diverges gets 1e50 everywhere, as vec_ops.c:292-296.  res: the
 * largest iteration count and the worst status.  nx even, V <= 16384. */
int tg_fm_propagator(tg_lattice* L, const tg_cg_params* cp, const int* mask, double* Dinv, tg_cg_result* res);

/* ---- dense matrix and determinant (tiny lattices) ------------------------ */
/* fermion_matrix (hmc.c:269-310) for the lattice's gauge field, row-major
 * complex: Md[(i*V + j)*2 + {0,1}] = M_ij with (M psi)_i = sum_j M_ij psi_j.
 * (The reference stores the same elements column-major for LAPACK.)  V <= 4096. */
int tg_dense_M(tg_lattice* L, double* Md);
/* determinant (hmc.c:314-336) as log|det M| and arg det M in (-pi, pi], for
 * nconf gauge fields A (double[nconf*V*2], or NULL for the lattice's own) by
 * one GPU LU factorisation with partial pivoting per field.  V <= 1024.
 * Leaves the lattice's gauge field at the last A. */
int tg_log_det(tg_lattice* L, int nconf, const double* A, double* logabs, double* phase);

/* ---- fermion-bag operator (vec_ops.c) ------------------------------------ */
/* fM / fM_transpose (vec_ops.c:96-174): the real, gauge-field-free staggered
 * operator with occupied sites (mask[s] != 0) acting as the identity and
 * skipped as neighbours; uses the lattice's m, mu and boundary conditions
 * (the reference's ANTISYMMETRIC build: both antiperiodic).  Host double[V]. */
int tg_fm_apply(tg_lattice* L, const int* mask, const double* in, double* out, int transpose);
/* cg_MdM (vec_ops.c:261-307): CG on fM^T fM from x = 0; the reference stops
 * at |r|^2 < 1e-30 (Thirring.h:42) within 10000 iterations (Thirring.h:43). */
int tg_cg_mdm_masked(tg_lattice* L, const tg_cg_params* cp, const int* mask, const double* b, double* x,
                     tg_cg_result* res);

/* ---- CG without allocation -------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * programs whose device memory is fully budgeted up front (a framework's
 * caching allocator owns the free memory) or that must not stall other
 * streams (cudaMalloc/cudaFree can synchronize the device).  Solves
 * M^dagger M x = b like tg_cg (FP64 solver only) on the calling thread's
 * current device, with no tg_lattice and no allocation of any kind: every
 * work vector lives in one fixed device array inside the library, sized for
 * lattices of at most 16384 sites (128 x 128); larger lattices get TG_E_ARG.
 * A_dev: gauge field double[nt*nx*2]; b_dev, x_dev: double2[nt*nx] on that
 * device; p->device is not used; stream may be NULL (the default stream).
 * The first call on a device looks up the array's device address.  No call
 * can run inside a stream capture: the solve reads its state back to the host
 * and synchronizes the stream every 16 iterations, so a call on a capturing
 * stream (or on the legacy default stream while another stream captures)
 * returns TG_E_ARG before it enqueues anything.  All calls share the array
 * and it keeps the previous call's contents, so calls that overlap on the GPU
 * race: order them (one stream, or synchronize between them). */
int tg_cg_noalloc(const tg_lattice_params* p, const tg_cg_params* cp, const void* A_dev, const void* b_dev,
                  void* x_dev, tg_cg_result* res, void* stream);

/* ---- batched chains ------------------------------------------------------
 * Many independent HMC chains (different NT x NX, m, g, mu, seed) advanced
 * by one persistent kernel launch per trajectory: each team -- one thread
 * block, or a thread-block cluster of 2 or 4 blocks on as many SMs -- runs
 * whole chain trajectories (hmc.c:671-746) taken from a work queue, largest
 * first.
 * The reference runs one chain per process; a batch replaces N such runs.
 * Random fields are the Philox streams of TG_RNG_PHILOX keyed by each chain's
 * seed, so chain k reproduces a tg_lattice trajectory with the same seed. */
typedef struct tg_batch tg_batch;

typedef struct {
  int nt, nx;               /* lattice of this chain                           */
  double m, g, mu;          /* its couplings                                   */
  int bc_t, bc_x;           /* TG_BC_*                                         */
  unsigned long long seed;  /* Philox key of this chain                        */
} tg_chain_params;

typedef struct {
  int nsteps;               /* leapfrog steps per trajectory                   */
  double tau;               /* trajectory length                               */
  int stochastic_term;      /* as tg_hmc_params                                */
  int use_graph;            /* launch through a cached CUDA graph              */
  int block;                /* kernel instance: 0 = the tuned one; 128, 256, 384 or 512 threads
                               per block (one block per chain); or an instance id as
                               tg_batch_autotune reports it (block * 100 + 10 * blocks
                               per chain, when a thread-block cluster of 2 or 4 blocks
                               runs each chain, + minimum resident blocks per SM,
                               + 100000 * S / 1024 when the cluster's blocks split up
                               to run the chains of at most S = 4096 or 9216 sites
                               one per block)                                      */
  tg_cg_params cg;          /* per-chain solver                                */
} tg_batch_params;

/* A starts at 0 for every chain. */
int tg_batch_create(const tg_chain_params* chains, int nchains, int device, tg_batch** out);
int tg_batch_destroy(tg_batch* B);
int tg_batch_size(const tg_batch* B, int* nchains, long long* total_sites);
/* gauge field of one chain: double[nt*nx*2] */
int tg_batch_set_gauge(tg_batch* B, int chain, const double* A);
int tg_batch_get_gauge(tg_batch* B, int chain, double* A);
/* Checkpoint of a whole batch: every chain's parameters, its Philox trajectory
 * counter, and the gauge fields.  Little-endian layout, byte offsets:
 *   0 char[8] "TGBATCH1"   8 int32 version (1)   12 int32 nchains
 *   16 int64 total sites
 *   24 + 56 i: chain i -- int32 nt, nx, bc_t, bc_x; double m, g, mu;
 *              uint64 seed, trajectory counter
 *   24 + 56 nchains: double A[total sites * 2], the chains' fields concatenated
 *   in chain order ([t][x][dir] each).
 * Loading needs a batch created with the same chains (same order and
 * parameters); a loaded batch continues bitwise as the saved one would. */
size_t tg_batch_checkpoint_size(const tg_batch* B);
int tg_batch_checkpoint_save(tg_batch* B, void* buf, size_t size);
int tg_batch_checkpoint_load(tg_batch* B, const void* buf, size_t size);
/* One trajectory of every chain; results[nchains] (cg_ms = device time of the
 * whole batch).  Returns the worst CG status over the chains. */
int tg_batch_trajectory(tg_batch* B, const tg_batch_params* p, tg_traj_result* results);
/* Times one trajectory with every compiled instance of the batch kernel
 * (threads per block x minimum resident blocks per SM, which trades registers
 * against occupancy, one block or a cluster of 2 or 4 blocks per chain, and
 * whether a cluster's blocks take the smallest chains one each),
 * with the chains' state saved and restored around every trial, and makes the
 * fastest the default (p->block = 0).  *best_block = the winner's instance id
 * (as for tg_batch_params.block);
 * *best_ms = its device time. */
int tg_batch_autotune(tg_batch* B, const tg_batch_params* p, int* best_block, double* best_ms);

#ifdef __cplusplus
}
#endif
#endif /* THIRRING_GPU_H */
