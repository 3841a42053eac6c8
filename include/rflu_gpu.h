/*
 * rflu_gpu.h -- C ABI of the GB300 (sm_103a) implementation of RocfluMP's
 * explicit residual-and-update path (thierrydaoud/Rocflu).
 *
 * The reference's Fortran driver calls one subroutine per piece of the path;
 * each entry point below names the subroutine it replaces (file:line in the
 * reference).  The Fortran host keeps owning t_region and all its arrays and
 * passes plain pointers (C_LOC) and sizes; nothing is transferred in
 * ownership.  Index arguments are 1-based Fortran ids, translated once at
 * rflu_gpu_create.  Real arrays use the reference's column-major layouts:
 *   cv(5,nCells), dv(3,nCells), rhs(5,nCells), gradCell(3,5,nCells),
 *   fn(4,nFaces) = (nx,ny,nz,|A|), fc(3,nFaces), cofg(3,nCells),
 *   xyzMoms(10,nCells) in XYZ_MOM_11..XYZ_MOM_44 order.
 *
 * Return codes: 0 = success; negative = usage or CUDA error (the message is
 * available from rflu_gpu_last_error); positive = numerical event reported
 * by the kernels (RFLU_EVENT_*), with details in rflu_status.  The library
 * never traps or aborts; the caller maps a nonzero code to ErrorStop.
 * A context is not re-entrant; all its work runs on one CUDA stream it owns.
 */
#ifndef RFLU_GPU_H
#define RFLU_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RFLU_OK 0
#define RFLU_ERR_ARG (-1)
#define RFLU_ERR_CUDA (-2)
#define RFLU_ERR_UNSUPPORTED (-3)
#define RFLU_ERR_STATE (-4)
#define RFLU_EVENT_NAN 1          /* invalid (NaN) cells after an update */
#define RFLU_EVENT_POSITIVITY 2   /* p <= 0 cells floored (RFLU_CheckPositivity) */

/* Precision of the device path. */
#define RFLU_PREC_FP64 0        /* all FP64, fused multiply-add allowed */
#define RFLU_PREC_FP64_EXACT 1  /* all FP64, reference evaluation order, no FMA: bit-exact with the CPU restatement */
#define RFLU_PREC_MIXED 2       /* FP32 state/gradients/fluxes, FP64 master cv, p/c recovery, checks, RK combination */

/* Boundary types, modfloflu/ModParameters.F90:396-441 */
#define RFLU_BC_INFLOW_TOTANG 10
#define RFLU_BC_INFLOW_VELTEMP 11
#define RFLU_BC_OUTFLOW 20
#define RFLU_BC_SLIPWALL 60
#define RFLU_BC_NOSLIPWALL_HFLUX 70
#define RFLU_BC_NOSLIPWALL_TEMP 71
#define RFLU_BC_FARFIELD 80
#define RFLU_BC_INJECTION 90
#define RFLU_BC_SYMMETRY 100      /* planar mirror patches: a face is an interior face to the cell's reflection */
#define RFLU_BC_PERIODIC 110      /* translational pairs: no boundary faces left (rflu_setup_build identifies them) */
/* Per-patch boundary values and switches (pPatch%mixt%vals(:,0) and
 * pPatch%mixt%switches, modfloflu/ModParameters.F90:452-511), uniform over
 * the patch: RFLU_BCDAT_N values and RFLU_BCSWI_N switches per patch, in
 * the reference's BCDAT_* / BCSWI_* order (1-based there, 0-based here):
 *   inflow TOTANG:  PTOT, TTOT, BETAH, BETAV, MACH; switches TYPE, FIXED
 *   inflow VELTEMP: U, V, W, T, P;                  switches TYPE
 *   farfield:       MACH, ATTACK, SLIP, PRESS, TEMP; switches CORR (must be 0)
 *   injection:      MFRATE, TEMP
 * Outflow keeps patchOutflowType / patchPout. */
#define RFLU_BCDAT_N 8
#define RFLU_BCSWI_N 2

/* The reference's setup products for one region, as RFLU_InitFlowSolver
 * leaves them (rocflu/RFLU_InitFlowSolver.F90:496,646,888-931):
 * RFLU_BuildFaceList, RFLU_BuildGeometry, RFLU_BuildC2CStencil,
 * RFLU_ComputeWtsC2C. */
typedef struct {
  int nCells;
  int nFaces;               /* interior faces, pGrid%nFaces */
  const int *f2c;           /* (2,nFaces), 1-based */
  const double *fn;         /* (4,nFaces) */
  const double *fc;         /* (3,nFaces) */
  const double *vol;        /* (nCells) */
  const double *cofg;       /* (3,nCells) */
  int nPatches;
  const int *patchFaceOff;  /* nPatches+1 offsets (0-based) into the patch-face arrays */
  const int *bf2c;          /* (nBFaces), 1-based, patch after patch */
  const double *bfn;        /* (4,nBFaces) */
  const double *bfc;        /* (3,nBFaces) */
  const int *patchBcType;   /* RFLU_BC_* */
  const int *patchOutflowType; /* outflow: BCOPT_SUPERSONIC 0, SUBSONIC 1, MIXED 2 */
  const double *patchPout;  /* outflow static pressure */
  const int *patchOrder;    /* pPatch%spaceOrder, 1 or 2 */
  /* C2C stencils (pGrid%c2cs(icg)%cellMembs) as CSR; ignored for ORDER 1 */
  const int *c2csOff;       /* nCells+1, 0-based offsets */
  const int *c2csMembs;     /* 1-based cell ids */
  const double *xyzMoms;    /* (10,nCells) */
  /* inflow, farfield and injection patches (may be NULL when there are none) */
  const double *patchVals;  /* (RFLU_BCDAT_N, nPatches) */
  const int *patchSwitches; /* (RFLU_BCSWI_N, nPatches) */
  /* translational periodic meshes (may be NULL: none): the centroid of each
   * face in its second cell's frame (= fc off the periods) and the
   * translation of each stencil member's image (0 off the periods), so that
   * a member's offset is cofg(member) - cofg(cell) + c2csShift */
  const double *fc2;        /* (3,nFaces) */
  const double *c2csShift;  /* (3,c2csOff[nCells]) */
  /* symmetry patches (may be NULL / 0: none; RFLU_ModSymmetryPeriodic's
   * virtual cells): a stencil member seen through the reflections across
   * one or more symmetry planes carries the index of that reflection
   * (-1: none) and, in c2csShift, the offset of its reflected centroid from
   * its own; its velocity is Q u with Q the reflection's 3x3 matrix, its
   * density and pressure its own. */
  const int *c2csXf;        /* (c2csOff[nCells]) */
  int nXf;
  const double *xfQ;        /* (3,3,nXf), row-major per reflection */
} rflu_grid_desc;

/* Numerics, the reference input deck keys (libfloflu/ReadNumericsSection.F90,
 * ReadTimestepSection.F90, ReadReferenceSection.F90). */
typedef struct {
  int spaceOrder;   /* ORDER: 1 or 2 */
  int spaceDiscr;   /* DISCR: 1 Roe, 3 HLLC, 4 AUSM+ */
  int reconst;      /* RECONST: 0 none, 1 WENO (simple) and 2 WENO-XYZ gradient smoothing with the simple
                       positivity limiter, 10 Barth-Jespersen (frame-invariant velocity), 11 Venkatakrishnan,
                       100 componentwise BJ */
  int rkScheme;     /* RKSCHEME: 1 classical RK4, 2 Wray RK3, 3 Euler */
  int piclBuild;    /* 1 when reproducing the reference built with PICL (its CMake default) */
  int precision;    /* RFLU_PREC_* */
  double cp, gamma; /* CP, GAMMA */
  double cfl, epsEntr, dissFact; /* CFL, ENTROPY, DISSFACT */
  double dtImposed, dtMinLimit;  /* TIMESTEP, DTMINLIMIT */
  int options;      /* RFLU_OPT_* bits of the device layout (no deck key; 0 = default) */
  int cReconstCells;          /* CRECONSTC: 0 none, 1 gradients constrained at wall and injection faces */
  double cReconstCellsWeight; /* CRECONSTCW: weight of the constraint rows (the reference's default is 1) */
} rflu_num_desc;

/* rflu_num_desc::options */
#define RFLU_OPT_UNTILED 1  /* mixed mode: never stage tiles in shared memory (the gather-based gradient kernels
                               that meshes too irregular for the tile plan take) */

typedef struct {
  long long nanCells;      /* RFLU_CheckValidity events */
  long long posFixCells;   /* RFLU_CheckPositivity energy-floor fixes */
  long long negPCells;     /* RFLU_EnforceBounds tiny-negative-pressure clamps */
  int firstBadCell;        /* 1-based reference id of the first NaN cell, 0 if none */
  int stepsDone;
  double time;             /* device-side current time after rflu_gpu_step */
  double dtMin;            /* last dtMin */
} rflu_status;

typedef struct rflu_gpu_ctx rflu_gpu_ctx;

/* Create the device mirror of one region: uploads geometry, renumbers cells
 * (Morton order of cofg) and builds the cell-centric CSR structures.
 * Call once after RFLU_InitFlowSolver (rocflu/RFLU_InitFlowSolver.F90:270-1065). */
int rflu_gpu_create(const rflu_grid_desc *grid, const rflu_num_desc *num, rflu_gpu_ctx **ctx);
int rflu_gpu_destroy(rflu_gpu_ctx *ctx);
const char *rflu_gpu_last_error(void);
/* The CUDA stream (cudaStream_t) the context launches on. */
void *rflu_gpu_stream(rflu_gpu_ctx *ctx);

/* cv(5,nCells) host -> device, then RFLU_SetVarsContWrapper
 * (libflu/RFLU_SetVarsContWrapper.F90:79-167) on the device. */
int rflu_gpu_upload_state(rflu_gpu_ctx *ctx, const double *cv);
/* cv(5,nCells), dv(3,nCells) device -> host; either may be NULL. */
int rflu_gpu_download_state(rflu_gpu_ctx *ctx, double *cv, double *dv);

/* RFLU_TimeStepInviscid + RFLU_MinimumTimeStep
 * (rocflu/RFLU_TimeStepInviscid.F90:75-333, rocflu/RFLU_MinimumTimeStep.F90:75-245):
 * dtMin of the current state at currentTime. */
int rflu_gpu_timestep(rflu_gpu_ctx *ctx, double currentTime, double *dtMin);

/* One stage of RungeKuttaMP (libfloflu/RungeKuttaMP.F90:148-508): RKInitMP,
 * CellGradientsMP, ConvectiveFluxesMP, RKUpdateMP, RFLU_SetVarsContWrapper,
 * AfterUpdateMP, with the given global dtMin. */
int rflu_gpu_rk_stage(rflu_gpu_ctx *ctx, int iStage, double dtMin);
/* RungeKuttaMP (libfloflu/RungeKuttaMP.F90:75-514): all stages. */
int rflu_gpu_runge_kutta(rflu_gpu_ctx *ctx, double dtMin);
/* The stepping loop of RFLU_TimeStepping (rocflu/RFLU_TimeStepping.F90:429-628)
 * on the device: per step timestep, RungeKuttaMP, currentTime += dtMin, the
 * last step clipped to endTime (endTime <= 0: no clip).  *time in/out. */
int rflu_gpu_step(rflu_gpu_ctx *ctx, int nSteps, double *time, double endTime, int *stepsDone);
/* nSteps RungeKuttaMP calls with a fixed dtMin (no CFL evaluation). */
int rflu_gpu_run_fixed_dt(rflu_gpu_ctx *ctx, int nSteps, double dtMin);

/* One RK stage at the reference's subroutine granularity, so that the host
 * can change the residual between the fluxes and the update as
 * SourceTermsMP and PICL_Runge do (libfloflu/RungeKuttaMP.F90:209-348).
 * Per stage, in this order:
 *   rflu_gpu_cell_gradients(ctx)        CellGradientsMP(region)
 *       (libfloflu/CellGradientsMP.F90:75; modfloflu/ModInterfaces.F90:100-103)
 *   rflu_gpu_convective_fluxes(ctx)     ConvectiveFluxesMP(region)
 *       (libfloflu/ConvectiveFluxesMP.F90:73; ModInterfaces.F90:116-119):
 *       rhs = -diss + the face fluxes, kept on the device
 *   rflu_gpu_add_rhs(ctx, src, onDevice), any number of times:
 *       rhs += src, src(5,nCells) in the reference's cell order and the
 *       units of rhs (SourceTermsMP subtracts vol*S for a source density S);
 *       the sum is formed in FP64 and stored in the mode's residual type
 *   rflu_gpu_rk_update(ctx, iStage, dtMin)  RKUpdateMP(region,iReg,istage)
 *       (libfloflu/RkUpdateMP.F90:75; ModInterfaces.F90:210-214) +
 *       RFLU_SetVarsContWrapper + AfterUpdateMP; returns RFLU_EVENT_NAN like
 *       rflu_gpu_rk_stage
 * RKInitMP (cvOld = cv, diss = 0; RkInitMP.F90:74) needs no call: the
 * device keeps cv unchanged until the update.  Without source terms the
 * sequence leaves the state rflu_gpu_rk_stage leaves, bit for bit.  A call
 * out of this order (fluxes without gradients of the current state, a
 * source or an update without fluxes) returns RFLU_ERR_STATE; every other
 * entry point that changes the state or evaluates a residual ends the
 * sequence.  onDevice = 0: src is host memory, reusable when the call
 * returns; onDevice = 1: device memory on the context's device (or managed),
 * which must be complete before the call (it runs on the context's stream
 * and waits for no other). */
int rflu_gpu_cell_gradients(rflu_gpu_ctx *ctx);
int rflu_gpu_convective_fluxes(rflu_gpu_ctx *ctx);
int rflu_gpu_add_rhs(rflu_gpu_ctx *ctx, const double *src, int onDevice);
int rflu_gpu_rk_update(rflu_gpu_ctx *ctx, int iStage, double dtMin);
/* Read-outs of the sequence above in the reference's cell order: rhs(5,nCells)
 * after rflu_gpu_convective_fluxes (and any rflu_gpu_add_rhs), the limited
 * gradCell(3,5,nCells) after rflu_gpu_cell_gradients (zero at first order),
 * as region%mixt%rhs and region%mixt%gradCell hold them there (PICL_Runge
 * interpolates gradCell).  onDevice as for rflu_gpu_add_rhs; both return
 * once the data are in place. */
int rflu_gpu_get_rhs(rflu_gpu_ctx *ctx, double *rhs, int onDevice);
int rflu_gpu_get_grad(rflu_gpu_ctx *ctx, double *grad, int onDevice);

/* One residual evaluation, CellGradientsMP (libfloflu/CellGradientsMP.F90:75)
 * + ConvectiveFluxesMP (libfloflu/ConvectiveFluxesMP.F90:73), for the host
 * state cv(5,nCells): rhs(5,nCells) and the limited gradCell(3,5,nCells)
 * (grad may be NULL).  Leaves the context state untouched. */
int rflu_gpu_residual(rflu_gpu_ctx *ctx, const double *cv, double *rhs, double *grad);

/* Discrete adjoint of the same residual (no reference counterpart; it
 * differentiates rflu_gpu_residual): cvBar = (dR/dcv)^T rhsBar, through the
 * limiter's active branch.  Arrays (5,nCells).  In the mixed mode the flux,
 * reconstruction, limiter and cons -> prim Jacobians are FP32 (the last in
 * closed form: unlike the pressure recovery it differentiates, it has no
 * cancellation).  The eigen-frame velocity limiter (RECONST 10) is
 * differentiated through its active branch with the eigenvectors' first-
 * order perturbation (the tangent uses the same linearisation).  RECONST 1
 * and 2: the WENO averages are differentiated (weights included) and the
 * simple limiter through its branch (a zeroed gradient has no derivative);
 * the smoothing's transpose is a gather over the transposed stencil.
 * CRECONSTC 1: the constrained fit is differentiated through its planned
 * weights (constant constraint values at the walls; a burning injection
 * face's values through the pressure of the face's cell).  Periodic meshes: members and faces across
 * a period through their images' translations; symmetry patches: the
 * reflected members' values and gradients through their reflections, a
 * symmetry face's flux and limiter terms through the cell's reflection. */
int rflu_gpu_vjp(rflu_gpu_ctx *ctx, const double *cv, const double *rhsBar, double *cvBar);
/* Tangent of the same residual: rhsDot = (dR/dcv) cvDot (every limiter,
 * the WENO smoothing included). */
int rflu_gpu_jvp(rflu_gpu_ctx *ctx, const double *cv, const double *cvDot, double *rhsDot);
/* Diagnostics (no reference counterpart): the limiter's active branches at
 * the host state cv(5,nCells), the branches through which rflu_gpu_vjp and
 * rflu_gpu_jvp differentiate.  branches(10,nCells), per cell and variable k
 * (0..4): the active face as the index of the face among the cell's faces
 * in the reference's summation order (-1: the factor is 1), and the
 * 0-based reference id of the neighbour whose value is the active extreme
 * (-1: none).  RECONST 10 reports its velocity eigen-axes in k = 1..3, the
 * face index times 4 plus the side (1: largest increment, 2: smallest);
 * RECONST 1 and 2 report -2 as the face of density (k = 0) and pressure
 * (k = 4) where the simple limiter after the WENO smoothing zeroed the
 * gradient.  Second order only (first order: RFLU_ERR_UNSUPPORTED). */
int rflu_gpu_limiter_branches(rflu_gpu_ctx *ctx, const double *cv, int *branches);

/* Boundary-pressure functional J = sum over the faces of patch iPatch
 * (0-based) of p_f*|A_f|, p_f the limited second-order face pressure of the
 * owning cell, and its gradient dJ/dcv(5,nCells) (no reference counterpart). */
int rflu_gpu_patch_pressure(rflu_gpu_ctx *ctx, const double *cv, int iPatch, double *J, double *cvBar);
/* Time-unrolled discrete adjoint (no reference counterpart): from the host
 * state cv0(5,nCells), nSteps RungeKuttaMP steps with the fixed dtMin, and
 * the functional J = sum over n = 1..nSteps of dtMin * (the patch-pressure
 * functional of rflu_gpu_patch_pressure at the state after step n).  The
 * reverse sweep applies each stage's residual VJP with the RK combination
 * transposed; the state is checkpointed on the device every `every` steps
 * and each segment is recomputed from its checkpoint (the segment's stage
 * states only are held).  cvBar0(5,nCells) receives dJ/dcv0; with cvBar0
 * NULL only the forward sweep runs and J alone is returned.  stats[4] (may
 * be NULL): forward-sweep ms, reverse-sweep ms (recompute + adjoint), device
 * bytes held by the context and the call, number of checkpoints.  Every
 * precision mode (the mixed mode runs its own primal and FP32-Jacobian
 * adjoint).  Leaves the context state untouched. */
int rflu_gpu_unrolled_adjoint(rflu_gpu_ctx *ctx, const double *cv0, int nSteps, double dtMin, int every, int iPatch,
                              double *J, double *cvBar0, double *stats);

int rflu_gpu_status(rflu_gpu_ctx *ctx, rflu_status *status);

/* Diagnostics (no reference counterpart): runs nIter RK stages launch by
 * launch (no graph, after one untimed stage) with CUDA events between the
 * kernels on the context's stream and returns the mean duration in ms of
 * [0] gradient+limiter, [1] face fluxes, [2] gather+update, [3] time-step
 * reduction. */
int rflu_gpu_kernel_times(rflu_gpu_ctx *ctx, int nIter, double *ms);
/* Diagnostics (no reference counterpart): mean device time in ms, over nIter
 * repetitions after one untimed, of [0] one primal residual
 * (gradient+limiter, face fluxes, gather) and [1] one adjoint (rflu_gpu_vjp's
 * kernels) on the current device state. */
int rflu_gpu_adjoint_times(rflu_gpu_ctx *ctx, int nIter, double *ms);
/* Diagnostics: FP64 fused multiply-add rate of the current device in
 * TFLOP/s (independent FMA chains on every SM), the roof of FP64 kernels. */
int rflu_gpu_fp64_rate(double *tflops);
/* Diagnostics: compares the mixed mode's integer-pipe float<->double
 * conversions with the hardware conversions on n generated values (random
 * doubles, doubles near the float range, rounding ties, widened floats and
 * float midpoints) and returns the number of differing results. */
int rflu_gpu_check_conversions(long long n, unsigned long long seed, unsigned long long *mismatches);

/* Diagnostics: the mixed mode's FP64 reciprocal of rho and sound speed,
 * refined once by Newton-Raphson from FP32 seeds, against IEEE FP64 division
 * and square root on n generated values 2^e*m (m in [1,2), |e| <= 100):
 * maxRelErr[0] the largest relative error of the reciprocal, maxRelErr[1]
 * of the square root. */
int rflu_gpu_check_refinements(long long n, unsigned long long seed, double *maxRelErr);

/* Residual without any allocation (no counterpart in the reference).
 * Same result as rflu_gpu_residual (rhs only), for callers that cannot
 * allocate device memory at call time: hosts that reserve all device memory
 * up front under a fixed budget, and hosts that cannot let cudaMalloc or
 * cudaFree synchronize the device while their other streams run.
 *   cvDev  device (or managed) pointer to cv(5,nCells), reference order
 *   rhsDev device (or managed) pointer to rhs(5,nCells), written
 * The intermediates live in one file-scope static device array of 64 MiB,
 * which every GPU that loads the library keeps until the process exits;
 * meshes whose intermediates do not fit (about 200k hexahedra in FP64) are
 * rejected with RFLU_ERR_ARG and a message giving the bytes needed.  The
 * first call on a device looks up the array's device address (with that
 * device current); make that first call before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (other host threads,
 * other contexts on the same device) race and must be serialised by the
 * caller.  Both buffers must be device memory on the context's device (or
 * managed memory), and that device must be current: anything else is
 * refused with RFLU_ERR_ARG before a kernel is launched.
 * Ordering: the call runs on the context's stream (rflu_gpu_stream) and does
 * not wait for the caller's streams, so whatever writes cvDev must be
 * complete before the call (a device or stream synchronisation, or an event
 * the caller has waited on); rhsDev is complete when the call returns,
 * because it synchronises the context's stream before returning.  It calls
 * no cudaMalloc, cudaFree or allocating routine and leaves the context's own
 * state untouched (its cv, dv and status counters). */
int rflu_gpu_residual_static(rflu_gpu_ctx *ctx, const double *cvDev, double *rhsDev);

/* ------------------------------------------------------------------------ */
/* Host set-up: builds the reference's setup products from a raw mesh, for   */
/* hosts that do not run RFLU_InitFlowSolver.  Reproduces RFLU_BuildFaceList */
/* numbering (modflu/RFLU_ModFaceList.F90:784-1585), RFLU_BuildGeometry      */
/* (modflu/RFLU_ModGeometry.F90:307-700), RFLU_BuildC2CStencil               */
/* (modflu/RFLU_ModStencilsCells.F90:750-1440) and RFLU_ComputeWtsC2C        */
/* (modflu/RFLU_ModWeights.F90:1025-1915).                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nVert, nCells, nVertPerCell;  /* 4 tetrahedra or 8 hexahedra */
  const double *xyz;                /* (3,nVert) */
  const int *c2v;                   /* (nVertPerCell,nCells), 1-based, Rocflu local vertex order */
  int nPatches;
  const int *patchFaceOff;          /* nPatches+1 */
  const int *bf2v;                  /* (4,nBFaces), 1-based, 0 in slot 4 for triangles */
  /* translational periodic patch pairs (may be NULL: none): the patches'
   * RFLU_BC_* types and the 0-based related patch of each BC_PERIODIC (110)
   * patch (RELPATCH), -1 otherwise */
  const int *patchBcType;
  const int *patchRelated;
} rflu_mesh_desc;

typedef struct rflu_setup rflu_setup;

/* spaceOrder > 1 also builds the C2C stencils and their moments. */
int rflu_setup_build(const rflu_mesh_desc *mesh, int spaceOrder, rflu_setup **setup);
/* Fills the geometry/stencil fields of grid (pointers into setup-owned
 * memory, valid until rflu_setup_destroy); patch boundary data stay the
 * caller's to set. */
int rflu_setup_grid(rflu_setup *setup, rflu_grid_desc *grid);
int rflu_setup_destroy(rflu_setup *setup);
/* The boundary-face stencil of CRECONSTC 1 (RFLU_AddBFaces + RFLU_SortBFaces,
 * modflu/RFLU_ModStencilsUtils.F90:134-298,1501-1585, at most 9 faces per
 * cell) of a grid description (its stencils, boundary faces and patch
 * types): off (nCells+1) and faces (off[nCells] entries, 0-based boundary
 * face index, patch after patch, nearest first); faces may be NULL. */
int rflu_setup_bface_stencil(const rflu_grid_desc *grid, int *off, int *faces);

#ifdef __cplusplus
}
#endif
#endif
