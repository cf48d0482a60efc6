/*
 * CPU FP64 oracle for the CATHY FLOW3D hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This header belongs to the oracle: a serial, double-precision restatement
 * of the reference Fortran (CATHY, vendored by pyCATHY under
 * pyCATHY/tests/weil_exemple/my_cathy_prj/src/).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product library never links or calls it.
 *
 * Parity pins: the oracle reproduces the reference's stored outputs of the
 * weill example (examples/SSHydro/weill_exemple/output: grid3d, the NTERM
 * line of risul, and the first nonlinear iteration of iter/risul), see
 * tests/test_oracle_golden.py.
 *
 * Array conventions follow the reference: node, element and zone ids are
 * 1-based; per-(layer,zone) soil tables are indexed (zone-1)*nstr+(layer-1).
 */
#ifndef CATHY_ORACLE_H
#define CATHY_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_dem {
  int32_t nrow, ncol;          /* DEM cells (rows north->south)            */
  double delta_x, delta_y;     /* cell sizes                               */
  double west, south, factor;  /* origin and elevation multiplier          */
  const double* dem;           /* nrow*ncol, row-major, 0 = inactive cell  */
  const int32_t* zone;         /* nrow*ncol zone ids (1-based) or NULL      */
  int32_t nstr;                /* number of layers                         */
  const double* zratio;        /* nstr layer thickness fractions           */
  double base;                 /* depth scale for ZRATIO                   */
  int32_t ivert;               /* GEN3D vertical mode (0..4, 3 needs depth)*/
} orc_dem_t;

typedef struct orc_soil {
  int32_t nzone;
  /* per (layer,zone): index (zone-1)*nstr + (layer-1) */
  const double *permx, *permy, *permz, *elstor, *poros, *vgn, *vgrmc, *vgpsat;
  double pmin, scf;
  int32_t kslope;   /* 0 or 1 */
  double tolksl;
  /* Feddes root-water uptake (datin.f:424-428, etran.f): nveg rows of
   * PCANA, PCREF, PCWLT, ZROOT, PZ, OMGC; root_map = input/root_map
   * (nrow*ncol, row-major like the DEM) or NULL for vegetation type 1
   * everywhere.  Needed only when scf > 0. */
  int32_t nveg;
  const double* feddes;
  const double* root_map;
} orc_soil_t;

typedef struct orc_parm {
  int32_t iopt, lump, isolv, itmxcg, ituns, ituns1, ituns2, l2norm, nlrelx;
  int32_t isimgr;   /* 1 = subsurface only (PONDH_MIN forced to 1e10) */
  double tetaf, toluns, tolswi, ernlmx, tolcg, omega;
  double deltat, dtmin, dtmax, tmax, dtmaga, dtmagm, dtreds, dtredm;
  double pondh_min;
  int32_t precond;  /* Picard linear solver: 0 = IC(0)-PCG (SYMSLV), 1 = Jacobi-PCG */
  int32_t isfcvg;   /* 1: nonlinear convergence also needs the seepage-face
                       exit points to stay put (ISFCVG, datin.f:110) */
} orc_parm_t;

typedef struct orc_bc {
  int32_t hspatm, ieto, natm;  /* atmospheric series: natm records        */
  const double* atmtim;        /* natm times                              */
  const double* atminp;        /* natm * (hspatm ? 1 : nnod) rates [L/T]  */
  int32_t np; const int32_t* contp; const double* presc; /* non-atm Dirichlet */
  int32_t nq; const int32_t* contq; const double* q;     /* non-atm Neumann   */
  int32_t indp; double wtposition; const double* pinit;  /* initial condition */
  /* seepage faces (input/sfbc, sfvone.f): nsf faces, sfnum[f] nodes each,
   * sfnod = the faces' 1-based node lists one after another, each face
   * ordered by descending elevation */
  int32_t nsf; const int32_t* sfnum; const int32_t* sfnod;
} orc_bc_t;

/* One record per nonlinear iteration (the reference's `iter` file). */
typedef struct orc_iter_rec {
  int32_t nstep, iter, niter, ikmax;
  double deltat, time, pl2, pinf, pnew_ik, pold_ik, fl2, finf, lin_err, lin_res;
} orc_iter_rec_t;

/* One record per accepted time step (the reference's `mbeconv` file). */
typedef struct orc_step_rec {
  int32_t nstep, iter, nitert, nback;
  double deltat, time, store1, store2, dstore, cdstor, vin, cvin, vout, cvout,
         erras, errel, cerras, caeras;
  double sfflw;    /* seepage-face flux SFFLW of the step (fluxmb.f:46-60) */
  double vnd, vnn; /* non-atmospheric Dirichlet / Neumann volumes of the step */
} orc_step_rec_t;

void* orc_create(const orc_dem_t* dem, const orc_soil_t* soil,
                 const orc_parm_t* parm, const orc_bc_t* bc);
void  orc_destroy(void* h);

/* sizes: n, nt, nnod, ntri, nterm (for the selected IOPT storage) */
void orc_sizes(void* h, int32_t* out5);
/* mesh arrays (copies): x,y,z (n each), tetra (5*nt, as after RIORD for
 * IOPT=1), topol (n+1), ja (nterm), arenod (nnod), volnod (n) */
void orc_get_mesh(void* h, double* x, double* y, double* z, int32_t* tetra,
                  int32_t* topol, int32_t* ja, double* arenod, double* volnod);
/* tetra exactly as GEN3D writes grid3d (before the tetrahedral RIORD) */
void orc_get_tetra_gen3d(void* h, int32_t* tetra);

/* run one time step (FLOW3D + back-steps) -> 0 converged, 1 no back-step
 * possible (simulation ends), 2 simulation already finished */
int32_t orc_step(void* h);
/* run to TMAX; returns number of accepted steps or -1 on failure */
int32_t orc_run(void* h, int32_t max_steps);
/* run only the first nonlinear iteration of the first time step */
void orc_first_iteration(void* h, orc_iter_rec_t* rec);

int32_t orc_num_iter_recs(void* h);
void orc_get_iter_recs(void* h, orc_iter_rec_t* out);
int32_t orc_num_step_recs(void* h);
void orc_get_step_recs(void* h, orc_step_rec_t* out);

void orc_get_state(void* h, double* pnew, double* time_dt2);  /* time, deltat */
/* QTRANIE (n values, 1-based node k at out[k-1]) of the current time step
 * and VEG_TYPE of the surface nodes (nnod values) */
void orc_get_qtranie(void* h, double* qtranie, int32_t* veg_type);
/* seepage-face state, one entry per face node in input order: SFEX (exit
 * point flags) and SFQ (back-calculated fluxes) */
void orc_get_seepage(void* h, int32_t* sfex, double* sfq);
void orc_set_state(void* h, const double* ptimep, double time, double deltat);

/* ---- fine-grained kernels on the current state (for unit parity) ---- */
/* assemble the Picard system at the current state: returns LHS (after BC, with
 * Dirichlet diagonals restored to the assembled value), RHS after BC, XT5 and
 * a Dirichlet mask (1 = Dirichlet). COEF arrays follow the symmetric upper
 * storage (topol/ja of IOPT=1). */
void orc_picard_system(void* h, double* coef1, double* tnoti, double* xt5,
                       int32_t* dirmask);
/* ASSPIC (asspic.f:9) with the reference's argument list: TETRA(5,NT) and
 * TETJA(4,4,NT) with 1-based contents, column-major LMASS(4,4), BI/CI/DI(4,NT),
 * PERMX/PERMY/PERMZ(MAXSTR,*); COEF1/COEF2/COEF4 are accumulated in place. */
void orc_asspic(int32_t nt, int32_t ntri, const int32_t* tetra, const int32_t* tetja,
                const double* lmass, double* coef1, double* coef2, double* coef4,
                const double* et1e, const double* pel, const double* permx,
                const double* permy, const double* permz, const double* ckrwe,
                const double* volu, const double* volur, const double* bi,
                const double* ci, const double* di, int32_t maxstr);
/* ASSPIC's inputs at the current state (after orc_picard_system): TETJA
 * (16*nt), LMASS (16), ET1E/PEL/CKRWE/VOLU/VOLUR (nt), PERMX/PERMY/PERMZ
 * (nstr*nzone, leading dimension nstr), BI/CI/DI (4*nt) */
void orc_asspic_inputs(void* h, int32_t* tetja, double* lmass, double* et1e, double* pel,
                       double* permx, double* permy, double* permz, double* ckrwe,
                       double* volu, double* volur, double* bi, double* ci, double* di);
/* nodal soil characteristics at heads psi (n): sw, ckrw, etai, et2 */
void orc_vg_nodal(void* h, const double* psi, double* sw, double* ckrw,
                  double* etai, double* et2);
/* solve with SYMSLV (IC(0)-PCG) on a given symmetric upper CSR system;
 * returns NITER, writes x, err, res */
int32_t orc_symslv(int32_t n, int32_t nterm, int32_t numdir,
                   const int32_t* noddir, const int32_t* ja,
                   const int32_t* topol, double* x, const double* b,
                   const double* coef1, int32_t itmxcg, double tolcg,
                   int32_t jacobi, double* err_res);
/* NSYSLV (ISOLV 0: ILU(0)-BiCGSTAB; -5: Jacobi-BiCGSTAB) on full CSR */
int32_t orc_nsyslv(int32_t isolv, int32_t n, int32_t nterm, int32_t numdir,
                   const int32_t* noddir, const int32_t* ja,
                   const int32_t* topol, double* x, const double* b,
                   const double* coef1, int32_t itmxcg, double tolcg,
                   double* err_res);

#ifdef __cplusplus
}
#endif
#endif
