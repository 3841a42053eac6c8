! rflu_gpu.f90 -- ISO_C_BINDING interface of librflu_gpu.so (rflu_gpu.h) for
! the RocfluMP Fortran solver.  A maintainer adds this module to the solver's
! sources and calls the library in place of the subroutines each interface
! names (the C header gives file:line in the reference for each).  The
! derived types repeat the C structs field for field; arrays cross as C_LOC
! of the solver's own arrays (cv(5,nCells), dv(3,nCells), rhs(5,nCells),
! gradCell(3,5,nCells), ...), nothing changes owner.  Arguments that may be
! NULL, or that may be device memory, are TYPE(C_PTR) passed by value.
! Every function returns RFLU_OK (0), a negative error code (message from
! RFLU_GPU_LastError) or a positive numerical event.
MODULE RFLU_ModGPU

  USE ISO_C_BINDING

  IMPLICIT NONE

  INTEGER(C_INT), PARAMETER :: RFLU_OK = 0, &
                               RFLU_ERR_ARG = -1, &
                               RFLU_ERR_CUDA = -2, &
                               RFLU_ERR_UNSUPPORTED = -3, &
                               RFLU_ERR_STATE = -4, &
                               RFLU_EVENT_NAN = 1, &
                               RFLU_EVENT_POSITIVITY = 2
  INTEGER(C_INT), PARAMETER :: RFLU_PREC_FP64 = 0, &
                               RFLU_PREC_FP64_EXACT = 1, &
                               RFLU_PREC_MIXED = 2
  INTEGER(C_INT), PARAMETER :: RFLU_BC_INFLOW_TOTANG = 10, &
                               RFLU_BC_INFLOW_VELTEMP = 11, &
                               RFLU_BC_OUTFLOW = 20, &
                               RFLU_BC_SLIPWALL = 60, &
                               RFLU_BC_NOSLIPWALL_HFLUX = 70, &
                               RFLU_BC_NOSLIPWALL_TEMP = 71, &
                               RFLU_BC_FARFIELD = 80, &
                               RFLU_BC_INJECTION = 90, &
                               RFLU_BC_SYMMETRY = 100, &
                               RFLU_BC_PERIODIC = 110
  INTEGER(C_INT), PARAMETER :: RFLU_BCDAT_N = 8, &
                               RFLU_BCSWI_N = 2
  INTEGER(C_INT), PARAMETER :: RFLU_OPT_UNTILED = 1

  TYPE, BIND(C) :: rflu_grid_desc
    INTEGER(C_INT) :: nCells
    INTEGER(C_INT) :: nFaces
    TYPE(C_PTR) :: f2c
    TYPE(C_PTR) :: fn
    TYPE(C_PTR) :: fc
    TYPE(C_PTR) :: vol
    TYPE(C_PTR) :: cofg
    INTEGER(C_INT) :: nPatches
    TYPE(C_PTR) :: patchFaceOff
    TYPE(C_PTR) :: bf2c
    TYPE(C_PTR) :: bfn
    TYPE(C_PTR) :: bfc
    TYPE(C_PTR) :: patchBcType
    TYPE(C_PTR) :: patchOutflowType
    TYPE(C_PTR) :: patchPout
    TYPE(C_PTR) :: patchOrder
    TYPE(C_PTR) :: c2csOff
    TYPE(C_PTR) :: c2csMembs
    TYPE(C_PTR) :: xyzMoms
    TYPE(C_PTR) :: patchVals
    TYPE(C_PTR) :: patchSwitches
    TYPE(C_PTR) :: fc2
    TYPE(C_PTR) :: c2csShift
    TYPE(C_PTR) :: c2csXf
    INTEGER(C_INT) :: nXf
    TYPE(C_PTR) :: xfQ
  END TYPE rflu_grid_desc

  TYPE, BIND(C) :: rflu_num_desc
    INTEGER(C_INT) :: spaceOrder
    INTEGER(C_INT) :: spaceDiscr
    INTEGER(C_INT) :: reconst
    INTEGER(C_INT) :: rkScheme
    INTEGER(C_INT) :: piclBuild
    INTEGER(C_INT) :: precision
    REAL(C_DOUBLE) :: cp
    REAL(C_DOUBLE) :: gamma
    REAL(C_DOUBLE) :: cfl
    REAL(C_DOUBLE) :: epsEntr
    REAL(C_DOUBLE) :: dissFact
    REAL(C_DOUBLE) :: dtImposed
    REAL(C_DOUBLE) :: dtMinLimit
    INTEGER(C_INT) :: options
    INTEGER(C_INT) :: cReconstCells
    REAL(C_DOUBLE) :: cReconstCellsWeight
  END TYPE rflu_num_desc

  TYPE, BIND(C) :: rflu_status
    INTEGER(C_LONG_LONG) :: nanCells
    INTEGER(C_LONG_LONG) :: posFixCells
    INTEGER(C_LONG_LONG) :: negPCells
    INTEGER(C_INT) :: firstBadCell
    INTEGER(C_INT) :: stepsDone
    REAL(C_DOUBLE) :: time
    REAL(C_DOUBLE) :: dtMin
  END TYPE rflu_status

  TYPE, BIND(C) :: rflu_mesh_desc
    INTEGER(C_INT) :: nVert
    INTEGER(C_INT) :: nCells
    INTEGER(C_INT) :: nVertPerCell
    TYPE(C_PTR) :: xyz
    TYPE(C_PTR) :: c2v
    INTEGER(C_INT) :: nPatches
    TYPE(C_PTR) :: patchFaceOff
    TYPE(C_PTR) :: bf2v
    TYPE(C_PTR) :: patchBcType
    TYPE(C_PTR) :: patchRelated
  END TYPE rflu_mesh_desc

  INTERFACE

    ! ---- context --------------------------------------------------------------
    INTEGER(C_INT) FUNCTION rflu_gpu_create(grid, num, ctx) BIND(C, NAME='rflu_gpu_create')
      IMPORT :: C_INT, C_PTR, rflu_grid_desc, rflu_num_desc
      TYPE(rflu_grid_desc), INTENT(IN) :: grid
      TYPE(rflu_num_desc), INTENT(IN) :: num
      TYPE(C_PTR), INTENT(OUT) :: ctx
    END FUNCTION rflu_gpu_create

    INTEGER(C_INT) FUNCTION rflu_gpu_destroy(ctx) BIND(C, NAME='rflu_gpu_destroy')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION rflu_gpu_destroy

    TYPE(C_PTR) FUNCTION rflu_gpu_last_error() BIND(C, NAME='rflu_gpu_last_error')
      IMPORT :: C_PTR
    END FUNCTION rflu_gpu_last_error

    TYPE(C_PTR) FUNCTION rflu_gpu_stream(ctx) BIND(C, NAME='rflu_gpu_stream')
      IMPORT :: C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION rflu_gpu_stream

    ! ---- state transfer ---------------------------------------------------
    INTEGER(C_INT) FUNCTION rflu_gpu_upload_state(ctx, cv) BIND(C, NAME='rflu_gpu_upload_state')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*)
    END FUNCTION rflu_gpu_upload_state

    INTEGER(C_INT) FUNCTION rflu_gpu_download_state(ctx, cv, dv) BIND(C, NAME='rflu_gpu_download_state')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      TYPE(C_PTR), VALUE :: cv, dv
    END FUNCTION rflu_gpu_download_state

    ! ---- time step and stages ---------------------------------------------
    INTEGER(C_INT) FUNCTION rflu_gpu_timestep(ctx, currentTime, dtMin) BIND(C, NAME='rflu_gpu_timestep')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), VALUE :: currentTime
      REAL(C_DOUBLE), INTENT(OUT) :: dtMin
    END FUNCTION rflu_gpu_timestep

    INTEGER(C_INT) FUNCTION rflu_gpu_rk_stage(ctx, iStage, dtMin) BIND(C, NAME='rflu_gpu_rk_stage')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: iStage
      REAL(C_DOUBLE), VALUE :: dtMin
    END FUNCTION rflu_gpu_rk_stage

    INTEGER(C_INT) FUNCTION rflu_gpu_runge_kutta(ctx, dtMin) BIND(C, NAME='rflu_gpu_runge_kutta')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), VALUE :: dtMin
    END FUNCTION rflu_gpu_runge_kutta

    INTEGER(C_INT) FUNCTION rflu_gpu_step(ctx, nSteps, time, endTime, stepsDone) BIND(C, NAME='rflu_gpu_step')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nSteps
      REAL(C_DOUBLE), INTENT(INOUT) :: time
      REAL(C_DOUBLE), VALUE :: endTime
      INTEGER(C_INT), INTENT(OUT) :: stepsDone
    END FUNCTION rflu_gpu_step

    INTEGER(C_INT) FUNCTION rflu_gpu_run_fixed_dt(ctx, nSteps, dtMin) BIND(C, NAME='rflu_gpu_run_fixed_dt')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nSteps
      REAL(C_DOUBLE), VALUE :: dtMin
    END FUNCTION rflu_gpu_run_fixed_dt

    ! ---- one stage at subroutine granularity (CellGradientsMP,
    !      ConvectiveFluxesMP, the source-term slot, RKUpdateMP) ----------------
    INTEGER(C_INT) FUNCTION rflu_gpu_cell_gradients(ctx) BIND(C, NAME='rflu_gpu_cell_gradients')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION rflu_gpu_cell_gradients

    INTEGER(C_INT) FUNCTION rflu_gpu_convective_fluxes(ctx) BIND(C, NAME='rflu_gpu_convective_fluxes')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
    END FUNCTION rflu_gpu_convective_fluxes

    INTEGER(C_INT) FUNCTION rflu_gpu_add_rhs(ctx, src, onDevice) BIND(C, NAME='rflu_gpu_add_rhs')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      TYPE(C_PTR), VALUE :: src
      INTEGER(C_INT), VALUE :: onDevice
    END FUNCTION rflu_gpu_add_rhs

    INTEGER(C_INT) FUNCTION rflu_gpu_rk_update(ctx, iStage, dtMin) BIND(C, NAME='rflu_gpu_rk_update')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: iStage
      REAL(C_DOUBLE), VALUE :: dtMin
    END FUNCTION rflu_gpu_rk_update

    INTEGER(C_INT) FUNCTION rflu_gpu_get_rhs(ctx, rhs, onDevice) BIND(C, NAME='rflu_gpu_get_rhs')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      TYPE(C_PTR), VALUE :: rhs
      INTEGER(C_INT), VALUE :: onDevice
    END FUNCTION rflu_gpu_get_rhs

    INTEGER(C_INT) FUNCTION rflu_gpu_get_grad(ctx, grad, onDevice) BIND(C, NAME='rflu_gpu_get_grad')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      TYPE(C_PTR), VALUE :: grad
      INTEGER(C_INT), VALUE :: onDevice
    END FUNCTION rflu_gpu_get_grad

    ! ---- residual, its derivatives, functionals ------------------------------
    INTEGER(C_INT) FUNCTION rflu_gpu_residual(ctx, cv, rhs, grad) BIND(C, NAME='rflu_gpu_residual')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*)
      REAL(C_DOUBLE), INTENT(OUT) :: rhs(*)
      TYPE(C_PTR), VALUE :: grad
    END FUNCTION rflu_gpu_residual

    INTEGER(C_INT) FUNCTION rflu_gpu_vjp(ctx, cv, rhsBar, cvBar) BIND(C, NAME='rflu_gpu_vjp')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*), rhsBar(*)
      REAL(C_DOUBLE), INTENT(OUT) :: cvBar(*)
    END FUNCTION rflu_gpu_vjp

    INTEGER(C_INT) FUNCTION rflu_gpu_jvp(ctx, cv, cvDot, rhsDot) BIND(C, NAME='rflu_gpu_jvp')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*), cvDot(*)
      REAL(C_DOUBLE), INTENT(OUT) :: rhsDot(*)
    END FUNCTION rflu_gpu_jvp

    INTEGER(C_INT) FUNCTION rflu_gpu_limiter_branches(ctx, cv, branches) BIND(C, NAME='rflu_gpu_limiter_branches')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*)
      INTEGER(C_INT), INTENT(OUT) :: branches(*)
    END FUNCTION rflu_gpu_limiter_branches

    INTEGER(C_INT) FUNCTION rflu_gpu_patch_pressure(ctx, cv, iPatch, J, cvBar) BIND(C, NAME='rflu_gpu_patch_pressure')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv(*)
      INTEGER(C_INT), VALUE :: iPatch
      REAL(C_DOUBLE), INTENT(OUT) :: J
      TYPE(C_PTR), VALUE :: cvBar
    END FUNCTION rflu_gpu_patch_pressure

    INTEGER(C_INT) FUNCTION rflu_gpu_unrolled_adjoint(ctx, cv0, nSteps, dtMin, every, iPatch, J, cvBar0, stats) &
                   BIND(C, NAME='rflu_gpu_unrolled_adjoint')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      REAL(C_DOUBLE), INTENT(IN) :: cv0(*)
      INTEGER(C_INT), VALUE :: nSteps
      REAL(C_DOUBLE), VALUE :: dtMin
      INTEGER(C_INT), VALUE :: every
      INTEGER(C_INT), VALUE :: iPatch
      REAL(C_DOUBLE), INTENT(OUT) :: J
      TYPE(C_PTR), VALUE :: cvBar0
      TYPE(C_PTR), VALUE :: stats
    END FUNCTION rflu_gpu_unrolled_adjoint

    INTEGER(C_INT) FUNCTION rflu_gpu_status(ctx, status) BIND(C, NAME='rflu_gpu_status')
      IMPORT :: C_INT, C_PTR, rflu_status
      TYPE(C_PTR), VALUE :: ctx
      TYPE(rflu_status), INTENT(OUT) :: status
    END FUNCTION rflu_gpu_status

    ! ---- diagnostics ------------------------------------------------------
    INTEGER(C_INT) FUNCTION rflu_gpu_kernel_times(ctx, nIter, ms) BIND(C, NAME='rflu_gpu_kernel_times')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nIter
      REAL(C_DOUBLE), INTENT(OUT) :: ms(*)
    END FUNCTION rflu_gpu_kernel_times

    INTEGER(C_INT) FUNCTION rflu_gpu_adjoint_times(ctx, nIter, ms) BIND(C, NAME='rflu_gpu_adjoint_times')
      IMPORT :: C_INT, C_PTR, C_DOUBLE
      TYPE(C_PTR), VALUE :: ctx
      INTEGER(C_INT), VALUE :: nIter
      REAL(C_DOUBLE), INTENT(OUT) :: ms(*)
    END FUNCTION rflu_gpu_adjoint_times

    INTEGER(C_INT) FUNCTION rflu_gpu_fp64_rate(tflops) BIND(C, NAME='rflu_gpu_fp64_rate')
      IMPORT :: C_INT, C_DOUBLE
      REAL(C_DOUBLE), INTENT(OUT) :: tflops
    END FUNCTION rflu_gpu_fp64_rate

    INTEGER(C_INT) FUNCTION rflu_gpu_check_conversions(n, seed, mismatches) BIND(C, NAME='rflu_gpu_check_conversions')
      IMPORT :: C_INT, C_LONG_LONG
      INTEGER(C_LONG_LONG), VALUE :: n
      INTEGER(C_LONG_LONG), VALUE :: seed
      INTEGER(C_LONG_LONG), INTENT(OUT) :: mismatches
    END FUNCTION rflu_gpu_check_conversions

    INTEGER(C_INT) FUNCTION rflu_gpu_check_refinements(n, seed, maxRelErr) BIND(C, NAME='rflu_gpu_check_refinements')
      IMPORT :: C_INT, C_LONG_LONG, C_DOUBLE
      INTEGER(C_LONG_LONG), VALUE :: n
      INTEGER(C_LONG_LONG), VALUE :: seed
      REAL(C_DOUBLE), INTENT(OUT) :: maxRelErr(*)
    END FUNCTION rflu_gpu_check_refinements

    ! ---- residual on caller-owned device buffers, no allocation -------------
    INTEGER(C_INT) FUNCTION rflu_gpu_residual_static(ctx, cvDev, rhsDev) BIND(C, NAME='rflu_gpu_residual_static')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: ctx
      TYPE(C_PTR), VALUE :: cvDev, rhsDev
    END FUNCTION rflu_gpu_residual_static

    ! ---- host set-up (face list, geometry, stencils, moments) ------------------
    INTEGER(C_INT) FUNCTION rflu_setup_build(mesh, spaceOrder, setup) BIND(C, NAME='rflu_setup_build')
      IMPORT :: C_INT, C_PTR, rflu_mesh_desc
      TYPE(rflu_mesh_desc), INTENT(IN) :: mesh
      INTEGER(C_INT), VALUE :: spaceOrder
      TYPE(C_PTR), INTENT(OUT) :: setup
    END FUNCTION rflu_setup_build

    INTEGER(C_INT) FUNCTION rflu_setup_grid(setup, grid) BIND(C, NAME='rflu_setup_grid')
      IMPORT :: C_INT, C_PTR, rflu_grid_desc
      TYPE(C_PTR), VALUE :: setup
      TYPE(rflu_grid_desc), INTENT(INOUT) :: grid
    END FUNCTION rflu_setup_grid

    INTEGER(C_INT) FUNCTION rflu_setup_destroy(setup) BIND(C, NAME='rflu_setup_destroy')
      IMPORT :: C_INT, C_PTR
      TYPE(C_PTR), VALUE :: setup
    END FUNCTION rflu_setup_destroy

    INTEGER(C_INT) FUNCTION rflu_setup_bface_stencil(grid, off, faces) BIND(C, NAME='rflu_setup_bface_stencil')
      IMPORT :: C_INT, C_PTR, rflu_grid_desc
      TYPE(rflu_grid_desc), INTENT(IN) :: grid
      INTEGER(C_INT) :: off(*)
      TYPE(C_PTR), VALUE :: faces
    END FUNCTION rflu_setup_bface_stencil

  END INTERFACE

CONTAINS

  ! The message of the last failed call on this thread, for ErrorStop.
  FUNCTION RFLU_GPU_LastError() RESULT(msg)
    CHARACTER(LEN=:), ALLOCATABLE :: msg
    CHARACTER(KIND=C_CHAR), POINTER :: c(:)
    TYPE(C_PTR) :: p
    INTEGER :: n

    p = rflu_gpu_last_error()
    msg = ''
    IF ( .NOT. C_ASSOCIATED(p) ) RETURN
    CALL C_F_POINTER(p, c, [4096])
    n = 0
    DO WHILE ( n < 4096 )
      IF ( c(n+1) == C_NULL_CHAR ) EXIT
      n = n + 1
    END DO
    ALLOCATE(CHARACTER(LEN=n) :: msg)
    msg = TRANSFER(c(1:n), msg)
  END FUNCTION RFLU_GPU_LastError

END MODULE RFLU_ModGPU
