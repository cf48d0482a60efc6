/*
 * cathy_gb300.h -- C ABI of the GB300-native CATHY subsurface solver.
 *
 * The library replaces the CPU routines of CATHY's FLOW3D hot path with
 * hand-written CUDA for sm_103a.  Two kinds of entry points are exported:
 *
 *  (1) Drop-ins for the reference's own Fortran subroutine boundaries, with
 *      the same arguments (host arrays, Fortran 1-based index contents,
 *      scalars by pointer so that an ISO_C_BINDING interface can pass them
 *      by reference):
 *        cathy_gb300_symslv   <- SYMSLV  (solscal-extended.f:4669)
 *        cathy_gb300_nsyslv   <- NSYSLV  (solscal-extended.f:3063), ISOLV 0/-5
 *        cathy_gb300_asspic   <- ASSPIC  (asspic.f:9)
 *
 *  (2) A handle API that owns the device state of one simulation or of a
 *      whole ensemble and advances it time step by time step.  One call of
 *      cathy_gb300_step replaces the body of the reference's time loop around
 *      its FLOW3D call (cathy_main.f:2882-3843: BC update, FLOW3D
 *      flow3d.f:8, back-stepping bkstep.f, mass balance masbal.f, TIMUPD
 *      timupd.f) for every member of the handle at once.
 *
 * All functions return 0 on success or a negative CATHY_GB300_E* code.  The
 * library never falls back to a CPU path: without a usable CUDA device every
 * compute entry point returns CATHY_GB300_ENODEV.
 */
#ifndef CATHY_GB300_H
#define CATHY_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define CATHY_GB300_OK 0
#define CATHY_GB300_ENODEV (-1)    /* no CUDA device / CUDA error          */
#define CATHY_GB300_EINVAL (-2)    /* invalid argument                     */
#define CATHY_GB300_EMESH (-3)     /* mesh construction failed             */
#define CATHY_GB300_ENOMEM (-4)    /* device allocation failed             */
#define CATHY_GB300_EUNSUP (-5)    /* option not supported                 */

/* ---- inputs (contents of a CATHY project's input files) --------------- */

/* prepro/dem + input/dem_parameters (read by datin.f:189-266) */
typedef struct cathy_dem {
  int32_t nrow, ncol;          /* DEM cells, row 1 = north                 */
  double delta_x, delta_y;     /* cell sizes                               */
  double west, south, factor;  /* origin, elevation multiplier             */
  const double* dem;           /* nrow*ncol row-major; 0 = inactive cell   */
  const int32_t* zone;         /* nrow*ncol zone ids (1-based) or NULL     */
  int32_t nstr;                /* layers                                   */
  const double* zratio;        /* nstr thickness fractions                 */
  double base;                 /* depth scale                              */
  int32_t ivert;               /* GEN3D vertical mode 0,1,2,4              */
} cathy_dem_t;

/* input/soil for IVGHU=0; tables indexed (zone-1)*nstr + (layer-1) */
typedef struct cathy_soil {
  int32_t nzone;
  const double *permx, *permy, *permz, *elstor, *poros, *vgn, *vgrmc, *vgpsat;
  double pmin, scf;
  int32_t kslope;              /* 0 analytical slopes; 1 chord slopes
                                  between PTOLD and PTNEW once they differ
                                  by TOLKSL (chpic1.f, chnew1.f)           */
  double tolksl;
  /* Feddes root-water uptake, ETRAN (etran.f:6-81), used when scf > 0:
     nveg rows of PCANA PCREF PCWLT ZROOT PZ OMGC (datin.f:424-428) and the
     input/root_map raster (nrow*ncol like the DEM, datin.f:221-233; NULL =
     vegetation type 1 everywhere).  The Picard right-hand side loses
     QTRANIE (bcpic.f:84-86); the Newton one does not (bcnew.f).           */
  int32_t nveg;
  const double* feddes;
  const double* root_map;
} cathy_soil_t;

/* input/parm keys (datin.f:81-117) */
typedef struct cathy_parm {
  int32_t iopt, lump, isolv, itmxcg, ituns, ituns1, ituns2, l2norm, nlrelx;
  int32_t isimgr;
  double tetaf, toluns, tolswi, ernlmx, tolcg, omega;
  double deltat, dtmin, dtmax, tmax, dtmaga, dtmagm, dtreds, dtredm;
  double pondh_min;
  int32_t precond;             /* Picard: 0 IC(0), 1 Jacobi, 2 column line */
  int32_t isfcvg;              /* 1: nonlinear convergence also needs the
                                  seepage-face exit points to stay put
                                  (ISFCVG, datin.f:110; flow3d.f:238-271) */
} cathy_parm_t;

/* input/atmbc, nansfdirbc, nansfneubc, ic */
typedef struct cathy_bc {
  int32_t hspatm, ieto, natm;
  const double* atmtim;        /* natm times                               */
  const double* atminp;        /* natm * (hspatm ? 1 : nnod) rates         */
  int32_t np; const int32_t* contp; const double* presc;
  int32_t nq; const int32_t* contq; const double* q;
  /* initial heads (inital.f:97-103): INDP 0 uniform pinit[0], 1 nodal
     pinit[n], 2 water table at the surface (icvhe.f), 3 water table
     WTPOSITION above each column's bottom node (icvhwt.f), 4 water table
     WTPOSITION below the surface (icvdwt.f)                                */
  int32_t indp; double wtposition; const double* pinit;
  /* seepage faces (input/sfbc as sfvone.f reads it, time-invariant): nsf
     faces of sfnum[f] nodes, sfnod = the 1-based node lists one after the
     other, each face by descending elevation.  Exit points start where the
     initial head is >= 1e-8 (sfinit.f) and move after every nonlinear
     iteration (extall.f); their back-calculated outflow enters VOUT
     (fluxmb.f, masbal.f).                                                  */
  int32_t nsf; const int32_t* sfnum; const int32_t* sfnod;
} cathy_bc_t;

typedef struct cathy_member {
  cathy_dem_t dem;
  cathy_soil_t soil;
  cathy_parm_t parm;
  cathy_bc_t bc;
} cathy_member_t;

/* solver options of a handle */
typedef struct cathy_opts {
  int32_t precision;           /* 0: FP64 everywhere; 1: FP32 matrix and
                                  Krylov inside FP64 residual/refinement   */
  int32_t device;              /* CUDA device ordinal                      */
  int32_t inner_maxit;         /* FP32 inner iterations per refinement     */
  double inner_tol;            /* FP32 inner relative tolerance (<=0: 1e-8) */
  int32_t verbose;
  int32_t graphs;              /* 1: run each Picard iteration of the FP32
                                  path as one CUDA graph launch (the PCG
                                  loop as a device-driven conditional node);
                                  0: launch kernel by kernel               */
} cathy_opts_t;

/* per nonlinear iteration record (the reference's `iter` file) */
typedef struct cathy_iter_rec {
  int32_t nstep, iter, niter, ikmax;
  double deltat, time, pl2, pinf, pnew_ik, pold_ik, fl2, finf, lin_err, lin_res;
} cathy_iter_rec_t;

/* per accepted time step record (the reference's `mbeconv` file) */
typedef struct cathy_step_rec {
  int32_t nstep, iter, nitert, nback;
  double deltat, time, store1, store2, dstore, cdstor, vin, cvin, vout, cvout,
         erras, errel, cerras, caeras;
  double sfflw;                /* seepage-face flux SFFLW (fluxmb.f:46-60)  */
  double vnd, vnn;             /* volumes through the non-atmospheric
                                  Dirichlet and Neumann nodes over the step,
                                  VNDIN+VNDOUT and VNNIN+VNNOUT (masbal.f) */
} cathy_step_rec_t;

/* ---- library ----------------------------------------------------------- */
int32_t cathy_gb300_version(void);
/* number of usable CUDA devices (0 when none) */
int32_t cathy_gb300_device_count(void);

/* ---- host-only mesh construction (no device needed) --------------------- */
/* Builds the mesh of a DEM exactly as the handle does (TRIANGOLI, GEN3D,
 * RIORD for IOPT=1, full CSR pattern).  Call once with NULL arrays to get
 * sizes (n, nt, nnod, ntri, nnz) in out5, then again with arrays of those
 * sizes: x,y,z (n), tetra (5*nt, 1-based), rowptr (n+1), cols (nnz), both
 * 0-based. */
int32_t cathy_gb300_mesh(const cathy_dem_t* dem, int32_t iopt, int32_t* out5,
                         double* x, double* y, double* z, int32_t* tetra,
                         int32_t* rowptr, int32_t* cols);

/* ---- handle API --------------------------------------------------------- */
/* The handle runs the reference's time loop around FLOW3D
 * (cathy_main.f:2882-3843: time-step control TIMUPD/BKSTEP, one FLOW3D call
 * per step at :3101, mass balance and output records) for one project or a
 * whole ensemble batched on one GPU. */
int32_t cathy_gb300_create(int32_t nmembers, const cathy_member_t* members,
                           const cathy_opts_t* opts, void** handle);
int32_t cathy_gb300_destroy(void* handle);
/* sizes of member m: n, nt, nnod, ntri, nnz (full CSR) */
int32_t cathy_gb300_sizes(void* handle, int32_t m, int32_t* out5);
/* advance every unfinished member by one accepted time step (with its
 * back-steps).  *nactive receives the number of members still running. */
int32_t cathy_gb300_step(void* handle, int32_t* nactive);
/* run every member to TMAX (or max_steps accepted steps) */
int32_t cathy_gb300_run(void* handle, int32_t max_steps, int32_t* nsteps);
/* state of member m: pressure heads (n), time, deltat, status
 * (0 running, 1 finished, 2 failed) */
int32_t cathy_gb300_get_state(void* handle, int32_t m, double* pnew,
                              double* time, double* deltat, int32_t* status);
int32_t cathy_gb300_set_state(void* handle, int32_t m, const double* ptimep,
                              double time, double deltat);
/* water saturation of member m at its current heads (n values, FP64): the
 * SW array that DETOUT writes to the sw output file (detout.f:44-45),
 * VGPNOT*Se(PNEW) + VGRMC/PNODI as CHNEW forms it */
int32_t cathy_gb300_get_saturation(void* handle, int32_t m, double* sw);
/* seepage faces of member m, one entry per face node in the order of
 * cathy_bc_t.sfnod: SFEX (1 = exit point) and the back-calculated flux SFQ
 * of the last iteration (extall.f, bkpic.f); EINVAL without faces */
int32_t cathy_gb300_get_seepage(void* handle, int32_t m, int32_t* sfex, double* sfq);
/* iteration records (one per Picard/Newton iteration: the `iter` file's
 * lines, conver.f:44-45) and step records (one per accepted step: the
 * `mbeconv` rows, cathy_main.f:3269-3273) of member m */
int32_t cathy_gb300_num_records(void* handle, int32_t m, int32_t* niter_recs,
                                int32_t* nstep_recs);
int32_t cathy_gb300_get_records(void* handle, int32_t m,
                                cathy_iter_rec_t* iter_recs,
                                cathy_step_rec_t* step_recs);
/* mesh of member m as built on the device: x,y,z (n), tetra (5*nt, 1-based,
 * node order as used for IOPT), rowptr (n+1, 0-based full CSR), cols (nnz,
 * 0-based) */
int32_t cathy_gb300_get_mesh(void* handle, int32_t m, double* x, double* y,
                             double* z, int32_t* tetra, int32_t* rowptr,
                             int32_t* cols);
/* Picard system of member m at its current state (LHS full CSR values before
 * Dirichlet masking, RHS after BCs, RHS before BCs, Dirichlet mask) */
int32_t cathy_gb300_picard_system(void* handle, int32_t m, double* vals,
                                  double* rhs, double* xt5, int32_t* dirmask);
/* restore every member to its initial condition (device-side copies) */
int32_t cathy_gb300_reset(void* handle);
/* live timing of the SpMV kernel: enable (1) / disable (0) resets the
 * counters; -1 only reads them.  Outputs: total device time of the timed
 * launches (ms; each launch timed on the device clock from its first
 * block's start to its last block's end, which also works inside the
 * graph's conditional PCG loop), launches, and their algorithmic bytes
 * (values+columns+row pointers+vectors). */
int32_t cathy_gb300_profile(void* handle, int32_t enable, double* spmv_ms,
                            int64_t* spmv_launches, double* spmv_bytes);
/* Schedule autotuner of the FP32 Picard path (no reference counterpart:
 * the reference runs serially).  On the handle's current state (every
 * running member; call it after the members have run a few steps) it times
 * the assembly kernel with its inputs read directly (mode 0) or staged
 * into shared memory by bulk copies (mode 1), 16 lanes per row, at 5, 6, 7
 * and 8 resident blocks per SM, and staged with 8 lanes per row (mode 2)
 * at 6, 8, 10 and 12 blocks of 128 threads, and the stream SpMV at 4, 6
 * and 8 resident blocks per SM or in its staged form (each warp's next
 * entry copied into shared memory while it multiplies the current one, 5
 * blocks per SM), nrep launches each,
 * and keeps the fastest; the choice is cached per (GPU, rows size class),
 * and nrep <= 0 reuses a cached choice when there is one.  sched[4]
 * receives (assembly blocks/SM, SpMV blocks/SM, assembly mode 0/1/2, SpMV
 * staged 0/1),
 * ms[2] their best mean ms.  The assembly variants give bit-identical
 * systems; the SpMV grid only regroups its FP32 dot products.
 * CATHY_GB300_EUNSUP outside the FP32 Picard path with the column-line
 * preconditioner. */
int32_t cathy_gb300_autotune(void* handle, int32_t nrep, int32_t* sched, double* ms);
/* Forces a schedule: assembly mode asm_staged 0 or 1 with blocks/SM in
 * {5, 6, 7, 8}, or 2 with {6, 8, 10, 12}; SpMV blocks/SM in 1..8 and
 * spmv_staged 0/1 (the staged form, which runs at 5 blocks/SM, is used for
 * work sets of more than two map entries per warp of a resident wave)
 * (defaults: mode 2 at 10 blocks/SM, SpMV 8, staged, on the FP32 Picard
 * path); CATHY_GB300_EUNSUP if a staged assembly is asked for and
 * unavailable. */
int32_t cathy_gb300_set_schedule(void* handle, int32_t asm_blocks, int32_t spmv_blocks,
                                 int32_t asm_staged, int32_t spmv_staged);
/* Phase timers of the nonlinear iterations in the nine buckets of the
 * reference's CPU summary (risul, cathy_main.f:3913-3950; accumulated in
 * picard.f:66-202): unsat characteristics, init of system matrices, local
 * assembly, RHS, global LHS, BC contributions, linear solver & residual,
 * Dirichlet resetting & DIFMAX, fluxes/mass balance/switching.  enable 1
 * starts them (zeroed) -- macro-iterations then run kernel by kernel with
 * CUDA events between the phases and NVTX ranges named after the buckets;
 * 0 stops them; -1 only reads.  out[0..n), n <= 9: GPU ms per bucket
 * (buckets whose work is fused into another kernel stay 0: the FP32 path
 * assembles matrix, RHS and BC terms in one kernel, bucket 3). */
int32_t cathy_gb300_phase_timers(void* handle, int32_t enable, double* out, int32_t n);
/* Times the FP32 Picard assembly (ASSPIC + RHSPIC + CFMATP + RHSGRV + BCPIC
 * fused, asspic.f:26-51) on the handle's current state: nrep launches over
 * the members that iterated in the last macro-iteration, between CUDA
 * events; the launches recompute the same system from unchanged inputs.
 * Outputs: mean ms per launch, the launch's algorithmic bytes (per row 74 B,
 * per surface row 16 B, per incidence 21 B (+4 B with a consistent mass
 * matrix), per matrix slot 9 B) and the rows assembled.  FP32 Picard path
 * only (CATHY_GB300_EUNSUP otherwise). */
int32_t cathy_gb300_time_assembly(void* handle, int32_t nrep, double* ms, double* bytes,
                                  int64_t* rows);
/* GPU time spent in the hot path (ms) since creation, and kernel launches */
int32_t cathy_gb300_stats(void* handle, double* gpu_ms, int64_t* launches,
                          int64_t* lin_iters, int64_t* nl_iters);

/* Timers of the time stepping (out[0..n), n <= 8): macro-iterations (one
 * nonlinear iteration of every member with work), CUDA graph launches, graph
 * builds, host preparation ms, device wait ms (launch + synchronise), host
 * decision ms, GPU ms of the hot path, GPU ms inside graph launches (CUDA
 * events around each launch); then, for n up to 72, 32 pairs (graph
 * launches, their GPU ms) binned by floor(log2(rows with work)). */
int32_t cathy_gb300_timers(void* handle, double* out, int32_t n);

/* ---- Fortran subroutine drop-ins ---------------------------------------- */
/* SYMSLV(IOUT,N,NTERM,NUMDIR,NITER,ITMXCG,TOLCG,RMIN,NODDIR,JA,TOPOL,PNEW,
 *        TNOTI,COEF1,COEF2,SCR): IC(0)-preconditioned CG on the symmetric
 * upper-triangular CSR system (diagonal first in each row, 1-based TOPOL/JA,
 * Dirichlet rows carrying the 1e-9*RMAX penalty).  PNEW receives the
 * solution; COEF2 and SCR are scratch as in the reference (COEF2 receives
 * the IC(0) factor).  ERR/RES (extra, may be NULL) receive the final
 * preconditioned-recursion and true residual norms. */
int32_t cathy_gb300_symslv(const int32_t* iout, const int32_t* n,
                           const int32_t* nterm, const int32_t* numdir,
                           int32_t* niter, const int32_t* itmxcg,
                           const double* tolcg, const double* rmin,
                           const int32_t* noddir, const int32_t* ja,
                           const int32_t* topol, double* pnew,
                           const double* tnoti, const double* coef1,
                           double* coef2, double* scr, double* err,
                           double* res);
/* NSYSLV restricted to ISOLV=0 (ILU(0)-BiCGSTAB, split preconditioning) and
 * ISOLV=-5 (Jacobi-BiCGSTAB) on the full nonsymmetric CSR (IA/JA/TOPOL). */
int32_t cathy_gb300_nsyslv(const int32_t* isolv, const int32_t* iout,
                           const int32_t* n, const int32_t* nterm,
                           const int32_t* numdir, const int32_t* noddir,
                           const int32_t* itmxcg, int32_t* niter,
                           const int32_t* ia, const int32_t* ja,
                           const int32_t* topol, const double* tolcg,
                           const double* rmin, const double* coef1,
                           double* coef2, double* pnew, const double* tnoti,
                           double* err, double* res);
/* ASSPIC(NT,NTRI,TETRA,TETJA,LMASS,COEF1,COEF2,COEF4,ET1E,PEL,PERMX,PERMY,
 *        PERMZ,CKRWE,ETAE,VOLU,VOLUR,BI,CI,DI): element assembly of the
 * Picard stiffness (COEF1) and mass (COEF2, COEF4) arrays, accumulated into
 * the caller's arrays as the reference does.  MAXSTR is the leading
 * dimension of PERMX/PERMY/PERMZ (CATHY.H), NTERM the length of COEF*. */
int32_t cathy_gb300_asspic(const int32_t* nt, const int32_t* ntri,
                           const int32_t* tetra, const int32_t* tetja,
                           const double* lmass, double* coef1, double* coef2,
                           double* coef4, const double* et1e,
                           const double* pel, const double* permx,
                           const double* permy, const double* permz,
                           const double* ckrwe, const double* etae,
                           const double* volu, const double* volur,
                           const double* bi, const double* ci,
                           const double* di, const int32_t* maxstr,
                           const int32_t* nterm);

/* ---- learned column-line preconditioner -------------------------------- */
/* No reference counterpart (the reference has no learned component); it is
 * the learned preconditioner wrapped inside the Picard PCG of the handle API
 * (SYMSLV's role, solscal-extended.f:4669).  A model is a small edge-wise
 * message-passing network (hidden width 64, BF16 weights, FP32
 * accumulation) that predicts per-edge weights omega_ij for the row-sum
 * compensation of the column-line (vertical tridiagonal block Jacobi)
 * factor: d'_i = a_ii + sum_{j horizontal} omega_ij a_ij.  Parameters are a
 * packed float vector of CATHY_GB300_LP_NPARAMS values:
 * W1 (64x16) | b1 (64) | W2 (64x64) | b2 (64) | w3 (64) | b3 (1). */
#define CATHY_GB300_LP_NPARAMS 5313
#define CATHY_GB300_LP_NPAIRS 4
/* params may be NULL (all zero) */
int32_t cathy_gb300_lp_create(const float* params, int32_t device, void** model);
int32_t cathy_gb300_lp_destroy(void* model);
/* get (may be NULL) / set (may be NULL) parameters; lr > 0 sets the Adam
 * learning rate; steps (may be NULL) receives the Adam steps taken */
int32_t cathy_gb300_lp_params(void* model, float* get, const float* set,
                              double lr, int64_t* steps);
/* One graph given on the host: full 0-based CSR of the Picard matrix (n
 * rows, nodes numbered layer by layer with nnod nodes per layer), Dirichlet
 * mask, nodal Ks, porosity and dSw/dpsi, the time step, and npairs Krylov
 * pairs (P, Q = A P; npairs x n).  train_steps = 0 evaluates the loss, the
 * network outputs (dprime: n, omega: nnz) and the parameter gradients
 * (grads: NPARAMS); train_steps > 0 first takes that many Adam steps. */
int32_t cathy_gb300_lp_eval(void* model, int32_t n, int32_t nnod,
                            const int32_t* rowptr, const int32_t* cols,
                            const float* vals, const uint8_t* dmask,
                            const float* ks, const float* pnodi,
                            const float* et2, float dt, int32_t npairs,
                            const float* P, const float* Q,
                            int32_t train_steps, double* loss, float* dprime,
                            float* omega, float* grads);

/* Attach a model to a handle (FP32 Picard path with the column-line
 * preconditioner, parm.precond = 2).  mode 1: train -- every Picard solve
 * stays plain, its first four Krylov pairs (p, q = A p) and matrices feed one
 * Adam step; mode 2: use -- members solve with the learned factor, every 8th
 * Picard iteration of a member is a plain probe, and a member keeps the
 * learned factor only while its mean PCG iteration count is not above the
 * plain one (plain column-line is the fallback; a column whose learned
 * pivots are not all positive also keeps the plain factor).  mode 0 or
 * model NULL detaches.  Kernel-by-kernel launches are used while a model is
 * attached. */
int32_t cathy_gb300_attach_learned(void* handle, void* model, int32_t mode);
/* out[0..n), n <= 6: learned solves, their PCG iterations, plain solves,
 * their PCG iterations (mode 2), training steps and last loss (mode 1) */
int32_t cathy_gb300_learned_stats(void* handle, double* out, int32_t n);

/* ---- allocation-free solve ----------------------------------------------- */
/* No counterpart in the reference: an extra entry point of this library for
 * callers that may not allocate device memory while they run (a driver whose
 * device memory belongs to a host framework's pool, or code that must not
 * allocate between time steps).  It runs the NSYSLV ISOLV=-5 solve of
 * cathy_gb300_nsyslv (Jacobi-preconditioned BiCGSTAB, same recurrences and
 * stopping rule) on arrays the caller already holds in DEVICE memory:
 * NODDIR (numdir, 1-based), JA/TOPOL (1-based full CSR), COEF1, TNOTI and
 * the output PNEW.  Scalars and the outputs NITER/ERR/RES are host pointers;
 * `stream` is a cudaStream_t (NULL = default stream).
 *
 * All workspace lives in one fixed device array compiled into the library,
 * so nothing is allocated: no cudaMalloc, cudaFree or allocating library
 * call.  That array is held on every GPU that loads the library until the
 * process exits, and it bounds n at CATHY_GB300_NOALLOC_MAXN rows; larger
 * systems are rejected with CATHY_GB300_EINVAL.  The first call on a device
 * looks up the array's device address.  The function waits for `stream` at
 * every iteration (it reads the convergence test back into host memory), so
 * it must not be called while that stream is being captured into a CUDA
 * graph.  Every call reuses the same array, so calls that overlap on the GPU
 * (from two streams or two host threads) race on it. */
#define CATHY_GB300_NOALLOC_MAXN 131072
int32_t cathy_gb300_nsyslv_noalloc(const int32_t* n, const int32_t* numdir,
                                   const int32_t* noddir_dev,
                                   const int32_t* itmxcg, int32_t* niter,
                                   const int32_t* ja_dev,
                                   const int32_t* topol_dev,
                                   const double* tolcg,
                                   const double* coef1_dev, double* pnew_dev,
                                   const double* tnoti_dev, double* err,
                                   double* res, void* stream);

#ifdef __cplusplus
}
#endif
#endif
