/*
 * CPU oracle for the RocfluMP explicit residual-and-update path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain FP64 C++ restatement of the
 * reference Fortran (thierrydaoud/Rocflu) used as the parity checker of the
 * GPU library and as the timed CPU baseline.  Nothing in the product links,
 * imports or calls it.  Every routine cites the reference file:line it
 * restates; the Fortran operation order is kept and the file is compiled with
 * -ffp-contract=off, matching the reference release flags (no FMA contraction).
 *
 * Parity status: the reference itself cannot be compiled here (no Fortran
 * compiler, no MPI).  One of its stored goldens lies on this path: the closed
 * gas-jump box (its tests/goldens/box/gas-jump/closed-creconst0/np2; HLLC,
 * second order, WENO-XYZ + the simple limiter, first-order slip walls, Wray
 * RK3, 569 steps), which this restatement reproduces to 6e-15 of each
 * field's maximum (the reference harness allows 1e-10).  Its other goldens
 * need periodic/symmetry patches, constrained gradients or particles, outside
 * this path; the Barth-Jespersen, Venkatakrishnan, Roe, AUSM+ and
 * outflow branches are pinned by the reference's property checks
 * (conservation to 1e-10, frame invariance of the BJ limiter to 1e-7) and
 * known-answer tests only.
 *
 * Indexing: all arrays use 0-based indices; layouts follow the reference
 * (column-major Fortran):  cv(5,nCells) -> cv[iv + 5*ic],
 * gradCell(3,5,nCells) -> grad[x + 3*(iv + 5*ic)], fn(4,nFaces), fc(3,nFaces).
 */
#ifndef RFLU_ORACLE_H
#define RFLU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Boundary condition types (modfloflu/ModParameters.F90:396-441). */
#define ORC_BC_INFLOW_TOTANG 10
#define ORC_BC_INFLOW_VELTEMP 11
#define ORC_BC_OUTFLOW 20
#define ORC_BC_SLIPWALL 60
#define ORC_BC_NOSLIPWALL_HFLUX 70
#define ORC_BC_NOSLIPWALL_TEMP 71
#define ORC_BC_FARFIELD 80
#define ORC_BC_INJECTION 90
#define ORC_BC_SYMMETRY 100
#define ORC_BC_PERIODIC 110
#define ORC_BCDAT_N 8
#define ORC_BCSWI_N 2

typedef struct {
  int nVert;
  int nCells;
  int nVertPerCell;        /* 4 = tetrahedra, 8 = hexahedra (pure meshes) */
  const double *xyz;       /* 3*nVert, interleaved x,y,z */
  const int *c2v;          /* nVertPerCell*nCells, 0-based, Rocflu local order */
  int nPatches;
  const int *patchFaceOff; /* nPatches+1 offsets into bf2v rows */
  const int *bf2v;         /* 4 per boundary face, -1 in slot 4 for triangles */
  const int *patchBcType;  /* ORC_BC_* */
  const int *patchOutflowType; /* 0 supersonic, 1 subsonic, 2 mixed */
  const double *patchPout; /* outflow static pressure */
  const int *patchOrder;   /* 1 or 2 */
  /* translational periodic patch pairs (BC_PERIODIC with RELPATCH): the
     0-based related patch of each patch, -1 for none; NULL: no periodic
     patches.  The two patches' faces are paired by their vertex
     coordinates, which differ by one translation per pair. */
  const int *patchRelated;
  /* pPatch%mixt%vals(:,0) and pPatch%mixt%switches of each patch in the
     reference's BCDAT_* / BCSWI_* order (ORC_BCDAT_N and ORC_BCSWI_N per
     patch); NULL when no patch needs them (inflow, farfield, injection) */
  const double *patchVals;
  const int *patchSwitches;
} orc_mesh_desc;

typedef struct {
  int spaceOrder;   /* 1 or 2 */
  int spaceDiscr;   /* 1 Roe, 3 HLLC, 4 AUSM+ */
  int reconst;      /* 0 none, 10 BJ (frame-invariant velocity), 11 Venkat, 100 BJ componentwise */
  int rkScheme;     /* 1 classical RK4, 2 Wray RK3, 3 Euler */
  int piclBuild;    /* 1: reference built with PICL (its default) -> energy slot holds p during fluxes */
  double cp, gamma;
  double cfl, epsEntr, dissFact;
  double dtImposed, dtMinLimit;
  int cReconstCells;          /* CRECONSTC: 1 constrains gradients at wall and injection faces */
  double cReconstCellsWeight; /* CRECONSTCW */
} orc_num_desc;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_mesh_desc *mesh, const orc_num_desc *num);
void orc_destroy(orc_ctx *c);

/* Sizes and setup products (face list, geometry, stencils, moments). */
int orc_nfaces(orc_ctx *c);
int orc_patch_nfaces(orc_ctx *c, int iPatch);
int orc_stencil_nnz(orc_ctx *c);
void orc_get_faces(orc_ctx *c, int *f2c, int *f2v, double *fn, double *fc);
void orc_get_cells(orc_ctx *c, double *vol, double *cofg);
void orc_get_patch(orc_ctx *c, int iPatch, int *bf2c, double *fn, double *fc);
void orc_get_stencil(orc_ctx *c, int *off, int *idx, double *moms);
/* CRECONSTC 1: the boundary-face stencil, off (nCells+1) and faces
 * (0-based boundary face index, patch after patch, nearest first); faces
 * may be NULL.  Built whatever CRECONSTC is (the reference always builds
 * it). */
void orc_get_bface_stencil(orc_ctx *c, int *off, int *faces);
/* Periodic meshes: fc2(3,nFaces) each face's centroid in its second cell's
 * frame (= fc off the periods) and stShift(3,nnz) the translation of each
 * stencil member's image (0 off the periods); either may be NULL. */
void orc_get_periodic(orc_ctx *c, double *fc2, double *stShift);
/* Symmetry patches: per stencil member the reflection it is seen through
 * (-1: none; else an index into the nXf velocity reflections, 9 values each,
 * row-major) and the offset of its reflected centroid from its own. */
int orc_n_reflections(orc_ctx *c);
void orc_get_symmetry(orc_ctx *c, int *stXf, double *stShift, double *xfQ);

/* State. cv(5,nCells) conserved; dv(3,nCells) = p,T,c. */
void orc_set_state(orc_ctx *c, const double *cv);
void orc_get_state(orc_ctx *c, double *cv, double *dv);
void orc_get_rhs(orc_ctx *c, double *rhs);
void orc_get_grad(orc_ctx *c, double *grad);

/* One residual evaluation (CellGradientsMP + ConvectiveFluxesMP) on a copy of
 * the current state; rhs(5,nCells) and limited gradCell(3,5,nCells). */
void orc_residual(orc_ctx *c, double *rhs, double *grad);

/* RFLU_TimeStepInviscid + RFLU_MinimumTimeStep; returns global dtMin. */
double orc_timestep(orc_ctx *c, double currentTime);
/* One RK stage of RungeKuttaMP with the given dtMin. */
void orc_rk_stage(orc_ctx *c, int iStage, double dtMin);
/* One RK stage in the pieces of RungeKuttaMP's stage body
 * (libfloflu/RungeKuttaMP.F90:209-348): RKInitMP; CellGradientsMP;
 * ConvectiveFluxesMP; rhs += src(5,nCells) (the SourceTermsMP / PICL_Runge
 * slot); RKUpdateMP + RFLU_SetVarsContWrapper + AfterUpdateMP.  Without a
 * source they are orc_rk_stage. */
void orc_rk_init(orc_ctx *c, int iStage);
void orc_cell_gradients(orc_ctx *c);
void orc_convective_fluxes(orc_ctx *c);
void orc_add_rhs(orc_ctx *c, const double *src);
void orc_rk_update(orc_ctx *c, int iStage, double dtMin);
/* Whole time steps: dt from the CFL condition each step, last step clipped to
 * endTime (endTime <= 0: no clip). Returns steps done; *time updated. */
int orc_run(orc_ctx *c, int nSteps, double *time, double endTime);
/* Whole time steps with a fixed dt (no CFL evaluation). */
void orc_run_fixed_dt(orc_ctx *c, int nSteps, double dt);
int orc_nstages(orc_ctx *c);

/* Replaces TIMESTEP (the imposed first time step) of the numerics. */
void orc_set_dt_imposed(orc_ctx *c, double dt);

/* Threads of the OpenMP loops (every call of this process); n <= 0 keeps
 * the current count.  orc_threads: the count the next loop will use (1 when
 * built without OpenMP).  Results do not depend on the count. */
void orc_set_threads(int n);
int orc_threads(void);

/* Positivity / bounds counters accumulated since creation. */
void orc_counters(orc_ctx *c, long long *posFix, long long *negP, long long *nan);

#ifdef __cplusplus
}
#endif
#endif
