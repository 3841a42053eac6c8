"""Host-side mirror of the reference's Fortran interface for this path, over
the C ABI of librflu_gpu.so (include/rflu_gpu.h).

A Region stands for the Fortran t_region of one grid region: it owns the
device mirror (rflu_gpu_ctx) and exposes the subroutines the solver driver
calls, under the reference's names:

  RFLU_TimeStepInviscid + RFLU_MinimumTimeStep -> Region.timestep
  RungeKuttaMP(regions)                          -> RungeKuttaMP(region, dtMin)
  RKInitMP/CellGradientsMP/ConvectiveFluxesMP/RKUpdateMP/AfterUpdateMP
                                                 -> Region.rk_stage(iStage, dtMin)
  CellGradientsMP(region)                        -> CellGradientsMP(region)
  ConvectiveFluxesMP(region)                     -> ConvectiveFluxesMP(region)
  SourceTermsMP / PICL_Runge's rhs changes       -> Region.add_rhs(src)
  RKUpdateMP(region, iReg, iStage)               -> RKUpdateMP(region, iReg, iStage, dtMin)
  the RFLU_TimeStepping loop                     -> Region.step(nSteps, time, endTime)

Arrays crossing the boundary use the reference layouts as (nCells, k)
C-order views: cv(5,nCells) column-major is cv[nCells, 5] row-major.

There is no CPU fallback: every call goes to the CUDA library, and loading
fails with an error when the library or a GPU is missing.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

PREC = {"fp64": 0, "fp64_exact": 1, "mixed": 2}
EVENT_NAN = 1

_LIB = None


class GridDesc(C.Structure):
    _fields_ = [("nCells", C.c_int), ("nFaces", C.c_int), ("f2c", C.POINTER(C.c_int)),
                ("fn", C.POINTER(C.c_double)), ("fc", C.POINTER(C.c_double)), ("vol", C.POINTER(C.c_double)),
                ("cofg", C.POINTER(C.c_double)), ("nPatches", C.c_int), ("patchFaceOff", C.POINTER(C.c_int)),
                ("bf2c", C.POINTER(C.c_int)), ("bfn", C.POINTER(C.c_double)), ("bfc", C.POINTER(C.c_double)),
                ("patchBcType", C.POINTER(C.c_int)), ("patchOutflowType", C.POINTER(C.c_int)),
                ("patchPout", C.POINTER(C.c_double)), ("patchOrder", C.POINTER(C.c_int)),
                ("c2csOff", C.POINTER(C.c_int)), ("c2csMembs", C.POINTER(C.c_int)),
                ("xyzMoms", C.POINTER(C.c_double)), ("patchVals", C.POINTER(C.c_double)),
                ("patchSwitches", C.POINTER(C.c_int)), ("fc2", C.POINTER(C.c_double)),
                ("c2csShift", C.POINTER(C.c_double)), ("c2csXf", C.POINTER(C.c_int)), ("nXf", C.c_int),
                ("xfQ", C.POINTER(C.c_double))]

BCDAT_N, BCSWI_N = 8, 2


def patch_values(case):
    """(nPatches, BCDAT_N) boundary values and (nPatches, BCSWI_N) switches of
    the case's patches (Patch.vals / Patch.switches, zero-padded)."""
    np_ = max(len(case.patches), 1)
    vals = np.zeros((np_, BCDAT_N), np.float64)
    sw = np.zeros((np_, BCSWI_N), np.int32)
    for i, p in enumerate(case.patches):
        v, w = tuple(getattr(p, "vals", ()) or ()), tuple(getattr(p, "switches", ()) or ())
        vals[i, :len(v)] = v
        sw[i, :len(w)] = w
    return vals, sw


class NumDesc(C.Structure):
    _fields_ = [("spaceOrder", C.c_int), ("spaceDiscr", C.c_int), ("reconst", C.c_int), ("rkScheme", C.c_int),
                ("piclBuild", C.c_int), ("precision", C.c_int), ("cp", C.c_double), ("gamma", C.c_double),
                ("cfl", C.c_double), ("epsEntr", C.c_double), ("dissFact", C.c_double),
                ("dtImposed", C.c_double), ("dtMinLimit", C.c_double), ("options", C.c_int),
                ("cReconstCells", C.c_int), ("cReconstCellsWeight", C.c_double)]


OPT_UNTILED = 1


class Status(C.Structure):
    _fields_ = [("nanCells", C.c_longlong), ("posFixCells", C.c_longlong), ("negPCells", C.c_longlong),
                ("firstBadCell", C.c_int), ("stepsDone", C.c_int), ("time", C.c_double), ("dtMin", C.c_double)]


class MeshDesc(C.Structure):
    _fields_ = [("nVert", C.c_int), ("nCells", C.c_int), ("nVertPerCell", C.c_int), ("xyz", C.POINTER(C.c_double)),
                ("c2v", C.POINTER(C.c_int)), ("nPatches", C.c_int), ("patchFaceOff", C.POINTER(C.c_int)),
                ("bf2v", C.POINTER(C.c_int)), ("patchBcType", C.POINTER(C.c_int)),
                ("patchRelated", C.POINTER(C.c_int))]


class RfluError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rflu error %d: %s" % (code, msg))
        self.code = code


EXPORTS = ("rflu_gpu_create", "rflu_gpu_destroy", "rflu_gpu_last_error", "rflu_gpu_stream",
           "rflu_gpu_upload_state", "rflu_gpu_download_state", "rflu_gpu_timestep", "rflu_gpu_rk_stage",
           "rflu_gpu_runge_kutta", "rflu_gpu_step", "rflu_gpu_run_fixed_dt", "rflu_gpu_cell_gradients",
           "rflu_gpu_convective_fluxes", "rflu_gpu_add_rhs", "rflu_gpu_rk_update", "rflu_gpu_get_rhs", "rflu_gpu_limiter_branches",
           "rflu_gpu_get_grad", "rflu_gpu_residual", "rflu_gpu_vjp",
           "rflu_gpu_jvp", "rflu_gpu_patch_pressure", "rflu_gpu_unrolled_adjoint", "rflu_gpu_status", "rflu_gpu_kernel_times", "rflu_gpu_residual_static",
           "rflu_gpu_adjoint_times", "rflu_gpu_fp64_rate", "rflu_gpu_check_conversions", "rflu_gpu_check_refinements", "rflu_setup_build", "rflu_setup_grid", "rflu_setup_bface_stencil",
           "rflu_setup_destroy")


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load librflu_gpu.so (building it first if needed).  Raises if the
    library cannot be built or loaded; there is no fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError("librflu_gpu.so is missing; run rocflu_gb300.build.build()")
    L = C.CDLL(_build.LIB)
    P, D, I = C.c_void_p, C.c_double, C.c_int
    DP = C.POINTER(C.c_double)
    L.rflu_gpu_create.argtypes = [C.POINTER(GridDesc), C.POINTER(NumDesc), C.POINTER(P)]
    L.rflu_gpu_destroy.argtypes = [P]
    L.rflu_gpu_last_error.restype = C.c_char_p
    L.rflu_gpu_stream.restype = P
    L.rflu_gpu_stream.argtypes = [P]
    L.rflu_gpu_upload_state.argtypes = [P, DP]
    L.rflu_gpu_download_state.argtypes = [P, DP, DP]
    L.rflu_gpu_timestep.argtypes = [P, D, DP]
    L.rflu_gpu_rk_stage.argtypes = [P, I, D]
    L.rflu_gpu_runge_kutta.argtypes = [P, D]
    L.rflu_gpu_step.argtypes = [P, I, DP, D, C.POINTER(I)]
    L.rflu_gpu_run_fixed_dt.argtypes = [P, I, D]
    L.rflu_gpu_cell_gradients.argtypes = [P]
    L.rflu_gpu_convective_fluxes.argtypes = [P]
    L.rflu_gpu_add_rhs.argtypes = [P, P, I]
    L.rflu_gpu_rk_update.argtypes = [P, I, D]
    L.rflu_gpu_get_rhs.argtypes = [P, P, I]
    L.rflu_gpu_get_grad.argtypes = [P, P, I]
    L.rflu_gpu_residual.argtypes = [P, DP, DP, DP]
    L.rflu_gpu_vjp.argtypes = [P, DP, DP, DP]
    L.rflu_gpu_jvp.argtypes = [P, DP, DP, DP]
    L.rflu_gpu_patch_pressure.argtypes = [P, DP, I, DP, DP]
    L.rflu_gpu_limiter_branches.argtypes = [P, DP, C.POINTER(C.c_int)]
    L.rflu_gpu_unrolled_adjoint.argtypes = [P, DP, I, D, I, I, DP, DP, DP]
    L.rflu_gpu_status.argtypes = [P, C.POINTER(Status)]
    L.rflu_gpu_kernel_times.argtypes = [P, I, DP]
    L.rflu_gpu_residual_static.argtypes = [P, P, P]
    L.rflu_gpu_adjoint_times.argtypes = [P, I, DP]
    L.rflu_gpu_fp64_rate.argtypes = [DP]
    L.rflu_gpu_check_conversions.argtypes = [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    L.rflu_gpu_check_refinements.argtypes = [C.c_longlong, C.c_ulonglong, DP]
    L.rflu_setup_build.argtypes = [C.POINTER(MeshDesc), I, C.POINTER(P)]
    L.rflu_setup_grid.argtypes = [P, C.POINTER(GridDesc)]
    L.rflu_setup_bface_stencil.argtypes = [C.POINTER(GridDesc), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.rflu_setup_destroy.argtypes = [P]
    for name in EXPORTS:
        if name not in ("rflu_gpu_last_error", "rflu_gpu_stream"):
            getattr(L, name).restype = C.c_int
    _LIB = L
    return L


def _check(rc, allow_events=False):
    if rc < 0 or (rc > 0 and not allow_events):
        msg = lib().rflu_gpu_last_error().decode() if rc < 0 else "numerical event"
        raise RfluError(rc, msg)
    return rc


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def num_desc(num, precision, options=0):
    return NumDesc(num.space_order, num.space_discr, num.reconst, num.rk_scheme, num.picl_build,
                   PREC[precision] if isinstance(precision, str) else int(precision), num.cp, num.gamma, num.cfl,
                   num.eps_entr, num.diss_fact, num.dt_imposed, num.dt_min_limit, int(options),
                   int(getattr(num, "c_reconst", 0)), float(getattr(num, "c_reconst_weight", 1.0)))


class Setup:
    """Reference setup products built on the host by rflu_setup_build
    (face list, geometry, C2C stencils, stencil moments)."""

    def __init__(self, case):
        L = lib()
        xyz = np.ascontiguousarray(case.xyz, np.float64)
        c2v = np.ascontiguousarray(case.c2v + 1, np.int32)
        off = np.zeros(len(case.patches) + 1, np.int32)
        for i, p in enumerate(case.patches):
            off[i + 1] = off[i] + len(p.bf2v)
        bf2v = np.concatenate([p.bf2v for p in case.patches]).astype(np.int32) + 1  # triangles: -1 -> 0
        bf2v = np.ascontiguousarray(bf2v)
        bct = np.array([p.bc_type for p in case.patches], np.int32)
        rel = np.array([getattr(p, "related", -1) for p in case.patches], np.int32)
        self._in = (xyz, c2v, off, bf2v, bct, rel)
        md = MeshDesc(xyz.shape[0], c2v.shape[0], c2v.shape[1], _p(xyz), _p(c2v, C.c_int), len(case.patches),
                      _p(off, C.c_int), _p(bf2v, C.c_int), _p(bct, C.c_int), _p(rel, C.c_int))
        h = C.c_void_p()
        _check(L.rflu_setup_build(C.byref(md), case.num.space_order, C.byref(h)))
        self.h = h
        g = GridDesc()
        _check(L.rflu_setup_grid(self.h, C.byref(g)))
        nc, nf = g.nCells, g.nFaces
        # periodic patches' faces are interior faces of the identified mesh:
        # the set-up's own patch offsets count them as none
        off = np.ctypeslib.as_array(g.patchFaceOff, (len(case.patches) + 1,)).copy()
        nb = int(off[-1])
        self.n_cells, self.n_faces = nc, nf
        self.f2c = np.ctypeslib.as_array(g.f2c, (nf, 2)).copy()
        self.fn = np.ctypeslib.as_array(g.fn, (nf, 4)).copy()
        self.fc = np.ctypeslib.as_array(g.fc, (nf, 3)).copy()
        self.vol = np.ctypeslib.as_array(g.vol, (nc,)).copy()
        self.cofg = np.ctypeslib.as_array(g.cofg, (nc, 3)).copy()
        self.patch_off = off
        if nb:
            self.bf2c = np.ctypeslib.as_array(g.bf2c, (nb,)).copy()
            self.bfn = np.ctypeslib.as_array(g.bfn, (nb, 4)).copy()
            self.bfc = np.ctypeslib.as_array(g.bfc, (nb, 3)).copy()
        else:  # every patch periodic
            self.bf2c, self.bfn, self.bfc = np.zeros(0, np.int32), np.zeros((0, 4)), np.zeros((0, 3))
        self.c2cs_off = np.ctypeslib.as_array(g.c2csOff, (nc + 1,)).copy()
        nnz = int(self.c2cs_off[-1])
        if nnz:
            self.c2cs = np.ctypeslib.as_array(g.c2csMembs, (nnz,)).copy()
            self.moms = np.ctypeslib.as_array(g.xyzMoms, (nc, 10)).copy()
        else:
            self.c2cs = np.zeros(0, np.int32)
            self.moms = np.zeros((nc, 10))
        # periodic meshes: face centroids in the second cells' frames and the
        # stencil members' image translations
        self.fc2 = np.ctypeslib.as_array(g.fc2, (nf, 3)).copy() if g.fc2 else None
        self.c2cs_shift = np.ctypeslib.as_array(g.c2csShift, (max(nnz, 1), 3))[:nnz].copy() if g.c2csShift else None
        # symmetry meshes: each stencil member's reflection (-1: none) and the
        # reflections' velocity matrices
        self.c2cs_xf = np.ctypeslib.as_array(g.c2csXf, (max(nnz, 1),))[:nnz].copy() if g.c2csXf else None
        self.xf_q = np.ctypeslib.as_array(g.xfQ, (g.nXf, 3, 3)).copy() if g.xfQ else None
        L.rflu_setup_destroy(self.h)
        self.h = None


def grid_desc(case, grid):
    """rflu_grid_desc of a case and its setup products (an object with the
    fields of Setup); returns the descriptor and the arrays it points into,
    which the caller keeps alive while the descriptor is used."""
    nc = int(grid.vol.shape[0])
    pt = np.array([p.bc_type for p in case.patches], np.int32)
    po = np.array([p.outflow_type for p in case.patches], np.int32)
    pp = np.array([p.p_out for p in case.patches], np.float64)
    pr = np.array([p.order for p in case.patches], np.int32)
    pv, psw = patch_values(case)
    arrs = dict(
        f2c=np.ascontiguousarray(grid.f2c, np.int32), fn=np.ascontiguousarray(grid.fn, np.float64),
        fc=np.ascontiguousarray(grid.fc, np.float64), vol=np.ascontiguousarray(grid.vol, np.float64),
        cofg=np.ascontiguousarray(grid.cofg, np.float64), off=np.ascontiguousarray(grid.patch_off, np.int32),
        bf2c=np.ascontiguousarray(grid.bf2c, np.int32), bfn=np.ascontiguousarray(grid.bfn, np.float64),
        bfc=np.ascontiguousarray(grid.bfc, np.float64), pt=pt, po=po, pp=pp, pr=pr,
        soff=np.ascontiguousarray(grid.c2cs_off, np.int32),
        smem=np.ascontiguousarray(grid.c2cs if len(grid.c2cs) else np.zeros(1), np.int32),
        moms=np.ascontiguousarray(grid.moms, np.float64), pv=pv, psw=psw)
    fc2 = getattr(grid, "fc2", None)
    shift = getattr(grid, "c2cs_shift", None)
    arrs["fc2"] = None if fc2 is None else np.ascontiguousarray(fc2, np.float64)
    arrs["shift"] = None if shift is None else np.ascontiguousarray(shift, np.float64)
    xf, xq = getattr(grid, "c2cs_xf", None), getattr(grid, "xf_q", None)
    arrs["xf"] = None if xf is None else np.ascontiguousarray(xf, np.int32)
    arrs["xq"] = None if xq is None else np.ascontiguousarray(xq, np.float64)
    a = arrs
    gd = GridDesc(nc, int(a["f2c"].shape[0]), _p(a["f2c"], C.c_int), _p(a["fn"]), _p(a["fc"]), _p(a["vol"]),
                  _p(a["cofg"]), len(case.patches), _p(a["off"], C.c_int), _p(a["bf2c"], C.c_int), _p(a["bfn"]),
                  _p(a["bfc"]), _p(a["pt"], C.c_int), _p(a["po"], C.c_int), _p(a["pp"]), _p(a["pr"], C.c_int),
                  _p(a["soff"], C.c_int), _p(a["smem"], C.c_int), _p(a["moms"]), _p(a["pv"]),
                  _p(a["psw"], C.c_int), None if a["fc2"] is None else _p(a["fc2"]),
                  None if a["shift"] is None else _p(a["shift"]),
                  None if a["xf"] is None else _p(a["xf"], C.c_int), 0 if a["xq"] is None else len(a["xq"]),
                  None if a["xq"] is None else _p(a["xq"]))
    return gd, arrs


def bface_stencil(case, grid=None):
    """The boundary-face stencil of CRECONSTC 1 (rflu_setup_bface_stencil):
    per cell (reference order) its wall and injection faces, nearest first,
    as 0-based boundary face indices; returns (off, faces)."""
    grid = Setup(case) if grid is None else grid
    gd, keep = grid_desc(case, grid)
    nc = int(grid.vol.shape[0])
    off = np.zeros(nc + 1, np.int32)
    _check(lib().rflu_setup_bface_stencil(C.byref(gd), _p(off, C.c_int), None))
    faces = np.zeros(max(int(off[-1]), 1), np.int32)
    _check(lib().rflu_setup_bface_stencil(C.byref(gd), _p(off, C.c_int), _p(faces, C.c_int)))
    return off, faces[:int(off[-1])]


class Region:
    """Device mirror of one region (t_region) in the given precision:
    'fp64', 'fp64_exact' or 'mixed'."""

    def __init__(self, case, precision="fp64", grid=None, options=0):
        """grid: the reference's setup products (an object with f2c (1-based),
        fn, fc, vol, cofg, bf2c (1-based), bfn, bfc, patch_off, c2cs_off,
        c2cs (1-based), moms); built by rflu_setup_build when omitted.
        options: rflu_num_desc::options bits (OPT_UNTILED)."""
        L = lib()
        self.case = case
        self.precision = precision
        if grid is None:
            grid = Setup(case)
        self.grid = grid
        nc = int(grid.vol.shape[0])
        self.n_cells = nc
        gd, self._desc_arrays = grid_desc(case, grid)
        self.nd = num_desc(case.num, precision, options)
        h = C.c_void_p()
        _check(L.rflu_gpu_create(C.byref(gd), C.byref(self.nd), C.byref(h)))
        self.h = h
        self.n_stages = {1: 4, 2: 3, 3: 1}[case.num.rk_scheme]
        if case.cv0 is not None:
            self.upload(case.cv0)

    def close(self):
        if getattr(self, "h", None):
            lib().rflu_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        """The CUDA stream handle (cudaStream_t) the region launches on."""
        return lib().rflu_gpu_stream(self.h)

    def upload(self, cv):
        cv = np.ascontiguousarray(cv, np.float64)
        assert cv.shape == (self.n_cells, 5)
        _check(lib().rflu_gpu_upload_state(self.h, _p(cv)))

    def download(self, cv_out=None, dv_out=None, with_dv=True):
        """cv (and dv unless with_dv is False: rflu_gpu_download_state with a
        NULL dv) in reference order."""
        cv = np.empty((self.n_cells, 5)) if cv_out is None else cv_out
        dv = None
        if with_dv:
            dv = np.empty((self.n_cells, 3)) if dv_out is None else dv_out
        _check(lib().rflu_gpu_download_state(self.h, _p(cv), _p(dv) if dv is not None else None))
        return cv, dv

    def timestep(self, current_time):
        dt = C.c_double()
        _check(lib().rflu_gpu_timestep(self.h, current_time, C.byref(dt)))
        return dt.value

    def rk_stage(self, istage, dt):
        return _check(lib().rflu_gpu_rk_stage(self.h, istage, dt), allow_events=True)

    def runge_kutta(self, dt):
        return _check(lib().rflu_gpu_runge_kutta(self.h, dt), allow_events=True)

    def step(self, n_steps, time=0.0, end_time=0.0):
        t = C.c_double(time)
        done = C.c_int()
        rc = _check(lib().rflu_gpu_step(self.h, n_steps, C.byref(t), end_time, C.byref(done)), allow_events=True)
        return done.value, t.value, rc

    def run_fixed_dt(self, n_steps, dt):
        return _check(lib().rflu_gpu_run_fixed_dt(self.h, n_steps, dt), allow_events=True)

    # one stage at the reference's subroutine granularity
    def cell_gradients(self):
        """CellGradientsMP (libfloflu/CellGradientsMP.F90:75) on the device state."""
        _check(lib().rflu_gpu_cell_gradients(self.h))

    def convective_fluxes(self):
        """ConvectiveFluxesMP (libfloflu/ConvectiveFluxesMP.F90:73): rhs kept on
        the device."""
        _check(lib().rflu_gpu_convective_fluxes(self.h))

    def add_rhs(self, src):
        """rhs += src (the SourceTermsMP / PICL_Runge slot): src a host
        (nCells, 5) array, or an int device address of one."""
        if isinstance(src, int):
            _check(lib().rflu_gpu_add_rhs(self.h, C.c_void_p(src), 1))
        else:
            s = np.ascontiguousarray(src, np.float64)
            assert s.shape == (self.n_cells, 5)
            _check(lib().rflu_gpu_add_rhs(self.h, s.ctypes.data_as(C.c_void_p), 0))

    def rk_update(self, istage, dt):
        """RKUpdateMP + RFLU_SetVarsContWrapper + AfterUpdateMP from the rhs."""
        return _check(lib().rflu_gpu_rk_update(self.h, istage, dt), allow_events=True)

    def get_rhs(self, out=None):
        """rhs(5,nCells) of the last convective_fluxes (and add_rhs): a host
        (nCells, 5) array, or written to an int device address."""
        if isinstance(out, int):
            _check(lib().rflu_gpu_get_rhs(self.h, C.c_void_p(out), 1))
            return None
        r = np.empty((self.n_cells, 5)) if out is None else out
        _check(lib().rflu_gpu_get_rhs(self.h, r.ctypes.data_as(C.c_void_p), 0))
        return r

    def get_grad(self, out=None):
        """gradCell(3,5,nCells) of the last cell_gradients as (nCells, 5, 3),
        or written to an int device address."""
        if isinstance(out, int):
            _check(lib().rflu_gpu_get_grad(self.h, C.c_void_p(out), 1))
            return None
        g = np.empty((self.n_cells, 5, 3)) if out is None else out
        _check(lib().rflu_gpu_get_grad(self.h, g.ctypes.data_as(C.c_void_p), 0))
        return g

    def residual(self, cv, with_grad=True):
        cv = np.ascontiguousarray(cv, np.float64)
        rhs = np.empty((self.n_cells, 5))
        grad = np.empty((self.n_cells, 5, 3)) if with_grad else None
        _check(lib().rflu_gpu_residual(self.h, _p(cv), _p(rhs), _p(grad) if with_grad else None))
        return rhs, grad

    def vjp(self, cv, rhs_bar):
        cv = np.ascontiguousarray(cv, np.float64)
        rb = np.ascontiguousarray(rhs_bar, np.float64)
        out = np.empty((self.n_cells, 5))
        _check(lib().rflu_gpu_vjp(self.h, _p(cv), _p(rb), _p(out)))
        return out

    def jvp(self, cv, cv_dot):
        cv = np.ascontiguousarray(cv, np.float64)
        cd = np.ascontiguousarray(cv_dot, np.float64)
        out = np.empty((self.n_cells, 5))
        _check(lib().rflu_gpu_jvp(self.h, _p(cv), _p(cd), _p(out)))
        return out

    def limiter_branches(self, cv):
        """(nCells, 5, 2) int: per variable the active face index and the
        reference id of the active extreme neighbour (rflu_gpu_limiter_branches)."""
        cv = np.ascontiguousarray(cv, np.float64)
        out = np.empty((self.n_cells, 5, 2), np.int32)
        _check(lib().rflu_gpu_limiter_branches(self.h, _p(cv), _p(out, C.c_int)))
        return out

    def patch_pressure(self, cv, ipatch, with_grad=True):
        cv = np.ascontiguousarray(cv, np.float64)
        J = C.c_double()
        g = np.empty((self.n_cells, 5)) if with_grad else None
        _check(lib().rflu_gpu_patch_pressure(self.h, _p(cv), ipatch, C.byref(J), _p(g) if with_grad else None))
        return J.value, g

    def unrolled_adjoint(self, cv0, n_steps, dt, every, ipatch, with_grad=True):
        """J = sum over the n_steps fixed-dt steps of dt * (patch-pressure
        functional after the step) and dJ/dcv0 by the checkpointed reverse
        sweep (rflu_gpu_unrolled_adjoint).  Returns (J, cv_bar0 or None,
        stats dict)."""
        cv0 = np.ascontiguousarray(cv0, np.float64)
        J = C.c_double()
        g = np.empty((self.n_cells, 5)) if with_grad else None
        st = np.zeros(4)
        _check(lib().rflu_gpu_unrolled_adjoint(self.h, _p(cv0), n_steps, dt, every, ipatch, C.byref(J),
                                               _p(g) if with_grad else None, _p(st)))
        return J.value, g, {"forward_ms": st[0], "reverse_ms": st[1], "device_bytes": int(st[2]),
                            "checkpoints": int(st[3])}

    def kernel_times(self, n_iter=10):
        """Mean ms per launch: grad+limiter, face flux, gather+update, dt."""
        ms = np.zeros(4)
        _check(lib().rflu_gpu_kernel_times(self.h, n_iter, _p(ms)))
        return ms

    def adjoint_times(self, n_iter=5):
        """Mean ms of one primal residual and of one VJP on the device state."""
        ms = np.zeros(2)
        _check(lib().rflu_gpu_adjoint_times(self.h, n_iter, _p(ms)))
        return ms

    def residual_static(self, cv_dev_ptr, rhs_dev_ptr):
        """rflu_gpu_residual_static on device buffers (integer device
        addresses of cv(5,nCells) and rhs(5,nCells) in reference order)."""
        _check(lib().rflu_gpu_residual_static(self.h, C.c_void_p(cv_dev_ptr), C.c_void_p(rhs_dev_ptr)))

    def status(self):
        s = Status()
        _check(lib().rflu_gpu_status(self.h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in Status._fields_}


def fp64_rate():
    """Measured FP64 FMA rate of the current GPU in TFLOP/s."""
    t = C.c_double()
    _check(lib().rflu_gpu_fp64_rate(C.byref(t)))
    return t.value


def check_conversions(n, seed=1):
    """Mismatches of the mixed mode's float<->double conversions against the
    hardware's over n generated values (0 expected)."""
    m = C.c_ulonglong()
    _check(lib().rflu_gpu_check_conversions(n, seed, C.byref(m)))
    return m.value


def check_refinements(n, seed=1):
    """Largest relative errors of the mixed mode's Newton-refined FP64
    reciprocal and square root against IEEE division and sqrt."""
    out = np.zeros(2)
    _check(lib().rflu_gpu_check_refinements(n, seed, _p(out)))
    return float(out[0]), float(out[1])


# --- the reference's subroutine names ---------------------------------------
def RungeKuttaMP(region, dt_min):
    """libfloflu/RungeKuttaMP.F90:75 -- all RK stages of one time step."""
    return region.runge_kutta(dt_min)


def RFLU_TimeStep(region, current_time):
    """rocflu/RFLU_TimeStepInviscid.F90:75 + rocflu/RFLU_MinimumTimeStep.F90:75."""
    return region.timestep(current_time)


def CellGradientsMP(region):
    """libfloflu/CellGradientsMP.F90:75 on the region's device state."""
    region.cell_gradients()


def ConvectiveFluxesMP(region):
    """libfloflu/ConvectiveFluxesMP.F90:73: the residual, kept on the device."""
    region.convective_fluxes()


def RKUpdateMP(region, i_reg, istage, dt_min):
    """libfloflu/RkUpdateMP.F90:75 (+ RFLU_SetVarsContWrapper, AfterUpdateMP);
    i_reg is the reference's region index, kept for the call's shape."""
    del i_reg
    return region.rk_update(istage, dt_min)


def CellGradientsMP_ConvectiveFluxesMP(region, cv):
    """libfloflu/CellGradientsMP.F90:75 then libfloflu/ConvectiveFluxesMP.F90:73:
    the residual rhs(5,nCells) and the limited gradCell(3,5,nCells)."""
    return region.residual(cv)
