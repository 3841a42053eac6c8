"""Problem set-ups: mesh, boundary patches, numerics and initial state.

The numeric keys mirror the reference input deck (libfloflu/
ReadNumericsSection.F90:110-129, ReadTimestepSection.F90:97-121,
ReadReferenceSection.F90:103-113): DISCR (1 Roe, 3 HLLC, 4 AUSM+), ORDER,
RECONST (0, 10 Barth-Jespersen with frame-invariant velocity limiting,
100 componentwise Barth-Jespersen, 11 Venkatakrishnan), RKSCHEME (1 classical
RK4, 2 Wray RK3, 3 Euler), CFL, ENTROPY, DISSFACT, TIMESTEP (imposed first
step), DTMINLIMIT, CP, GAMMA.  Boundary types follow modfloflu/
ModParameters.F90:401,413 (BC_OUTFLOW 20, BC_SLIPWALL 60); outflow TYPE 0 is
supersonic (extrapolation), 1 subsonic, 2 mixed (ModParameters.F90:501-503).
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import meshgen

BC_INFLOW_TOTANG = 10
BC_INFLOW_VELTEMP = 11
BC_OUTFLOW = 20
BC_SLIPWALL = 60
BC_NOSLIPWALL_HFLUX = 70
BC_NOSLIPWALL_TEMP = 71
BC_FARFIELD = 80
BC_INJECTION = 90
BC_SYMMETRY = 100
BC_PERIODIC = 110
BCOPT_SUPERSONIC, BCOPT_SUBSONIC, BCOPT_MIXED = 0, 1, 2

DISCR_ROE, DISCR_HLLC, DISCR_AUSM = 1, 3, 4
RECONST_NONE, RECONST_BJ, RECONST_VENKAT, RECONST_BJ_COMP = 0, 10, 11, 100
RECONST_WENO_SIMPLE, RECONST_WENO_XYZ = 1, 2
RK_CLASSICAL4, RK_WRAY3, RK_EULER = 1, 2, 3


@dataclass
class Patch:
    bf2v: np.ndarray
    bc_type: int = BC_SLIPWALL
    outflow_type: int = 0
    p_out: float = 0.0
    order: int = 1
    name: str = ""
    related: int = -1       # BC_PERIODIC: the 0-based related patch (RELPATCH)
    # inflow, farfield, injection: pPatch%mixt%vals(:,0) and switches in the
    # reference's BCDAT_* / BCSWI_* order (modfloflu/ModParameters.F90:452-511)
    vals: tuple = ()
    switches: tuple = ()


@dataclass
class Numerics:
    space_order: int = 2
    space_discr: int = DISCR_HLLC
    reconst: int = RECONST_BJ
    rk_scheme: int = RK_WRAY3
    picl_build: int = 1
    cp: float = 3.5
    gamma: float = 1.4
    cfl: float = 0.5
    eps_entr: float = 0.05
    diss_fact: float = 1.0
    dt_imposed: float = 1.0e-5
    dt_min_limit: float = 1.0e-10
    c_reconst: int = 0            # CRECONSTC: 1 constrains gradients at wall and injection faces
    c_reconst_weight: float = 1.0  # CRECONSTCW


@dataclass
class Case:
    name: str
    xyz: np.ndarray
    c2v: np.ndarray
    patches: list
    num: Numerics
    cv0: np.ndarray = None          # (nCells, 5) conserved state, cell order of c2v
    end_time: float = 0.0
    n_steps: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def n_cells(self):
        return self.c2v.shape[0]


def conserved(rho, u, v, w, p, gamma):
    """(rho, rho u, rho v, rho w, rho E) from primitive variables."""
    rho = np.asarray(rho, float)
    e = p / (rho * (gamma - 1.0)) + 0.5 * (u * u + v * v + w * w)
    return np.stack([rho, rho * u, rho * v, rho * w, rho * e], axis=1)


def _patches(mesh, kinds):
    out = []
    for p, k in zip(mesh["patches"], kinds):
        out.append(Patch(bf2v=p["bf2v"], name=p["name"], **k))
    return out


SLIP = {"bc_type": BC_SLIPWALL}


def gas_jump_closed(n=8, length=0.008, x_jump=0.0043, left=(1.2, 0.0, 101325.0), right=(0.97, 82700.0)):
    """The reference test suite's closed gas-jump box (tests/goldens/box/
    gas-jump/closed-creconst0; deck tests/templates/rectshktb.inp with its
    overrides): n^3 hexes on [0, length]^3, the hard-coded rectshktb state
    (utilities/init/RFLU_InitFlowHardCode.F90:839-910: rho, u, p = left for
    centroid x < x_jump, rho, p = right at rest beyond), slip walls on all six
    sides without an ORDER key, hence first order (spaceOrderBFaces,
    libflu/RFLU_InitInputValues.F90:195); HLLC, second order, WENO-XYZ
    (RECONST 2), no constrained gradients, Wray RK3, CFL 0.4, TIMESTEP 1e-9,
    DTMINLIMIT 2e-10, gamma 1.4, cp 1004.64, run to t = 1.05e-4."""
    mesh = meshgen.hex_box(n, n, n, hi=(length, length, length))
    num = Numerics(space_order=2, space_discr=DISCR_HLLC, reconst=RECONST_WENO_XYZ, rk_scheme=RK_WRAY3, cfl=0.4,
                   cp=1004.64, gamma=1.4, dt_imposed=1.0e-9, dt_min_limit=2.0e-10)
    patches = _patches(mesh, [dict(SLIP, order=1)] * 6)
    x = meshgen.cell_centers(mesh)[:, 0]
    inside = x < x_jump
    d = np.where(inside, left[0], right[0])
    u = np.where(inside, left[1], 0.0)
    p = np.where(inside, left[2], right[1])
    # the state as the hard-coded initialisation forms it: gamma from the gas
    # constant's round trip (MixtPerf_R_M / MixtPerf_G_CpR) and
    # d * MixtPerf_Eo_DGPUVW(d, g, p, u, v, w)
    gc = 8314.3 / (8314.3 / (num.cp - num.cp / num.gamma))
    g = num.cp / (num.cp - gc)
    z = np.zeros_like(d)
    cv0 = np.stack([d, d * u, z, z, d * (p / (d * (g - 1.0)) + 0.5 * (u * u))], axis=1)
    return Case("gas_jump_closed", mesh["xyz"], mesh["c2v"], patches, num, cv0, end_time=1.05e-4)


def gas_jump_periodic(n=8, length=0.008, x_jump=0.0043, left=(1.2, 0.0, 101325.0), right=(0.97, 82700.0)):
    """The reference test suite's periodic gas-jump box (tests/goldens/box/
    gas-jump/periodic/np1; the deck of gas_jump_closed with the golden's
    overrides, one region): the same n^3 hexes and hard-coded jump, periodic
    on all three axes (the harness's bc layout 'periodic', tests/
    rocpicl_tests/case.py:230-235: x-low/x-high, y-low/y-high and
    z-low/z-high translational pairs), so the jump at x_jump and the one at
    x = 0 = length both evolve; HLLC, second order, WENO-XYZ + the simple
    limiter, Wray RK3, CFL 0.4, TIMESTEP 1e-9, run to t = 1.05e-4."""
    c = gas_jump_closed(n, length, x_jump, left, right)
    for i, p in enumerate(c.patches):
        p.bc_type = BC_PERIODIC
        p.related = i ^ 1
        p.order = 1
    c.name = "gas_jump_periodic"
    return c


def gas_jump_symmetry(n=8, length=0.008, x_jump=0.0043, left=(1.2, 0.0, 101325.0), right=(0.97, 82700.0)):
    """The reference test suite's symmetry gas-jump box (tests/goldens/box/
    gas-jump/symmetry/np1): the periodic box's deck and jump with symmetry
    patches on all six sides (the harness's bc layout 'symmetry', tests/
    rocpicl_tests/case.py:241-242); a face on a symmetry patch is an interior
    face to the cell's reflection, so the patch order does not apply.  No
    wall or injection patch, so CRECONSTC 1 of the deck constrains nothing."""
    c = gas_jump_closed(n, length, x_jump, left, right)
    for p in c.patches:
        p.bc_type = BC_SYMMETRY
    c.name = "gas_jump_symmetry"
    return c


def mirror_box(n=6, axes=(0,), doubled=False, num=None, tets=False):
    """A smooth 3-D state (density and pressure bumps, all three velocity
    components nonzero) on n^3 hexes of [0,1]^3 with symmetry patches on the
    high sides of the given axes and first-order slip walls elsewhere; or,
    doubled, the box extended to [0,2] along those axes with the state
    mirrored about 1 (velocity component reversed) and slip walls all round.
    A symmetry patch stands for the mirrored half, so the two runs agree on
    [0,1]^3 wherever the scheme itself keeps the doubled box symmetric.
    tets: 6 tetrahedra per hex (no doubled form: the split is not mirror
    symmetric)."""
    mult = [2 if (doubled and a in axes) else 1 for a in range(3)]
    size = tuple(float(m) for m in mult)
    mesh = meshgen.tet_box(n, hi=size, jitter=0.1) if tets else meshgen.hex_box(n * mult[0], n * mult[1], n * mult[2], hi=size)
    if num is None:
        num = Numerics(space_order=2, space_discr=DISCR_HLLC, reconst=RECONST_WENO_XYZ, rk_scheme=RK_WRAY3, cfl=0.4)
    kinds = []
    for ip in range(6):
        ax, hi = ip // 2, ip % 2
        if hi and ax in axes and not doubled:
            kinds.append({"bc_type": BC_SYMMETRY, "order": 1})
        else:
            kinds.append(dict(SLIP, order=1))
    patches = _patches(mesh, kinds)
    c = meshgen.cell_centers(mesh)
    x, y, z = c[:, 0].copy(), c[:, 1].copy(), c[:, 2].copy()
    sgn = np.ones((len(x), 3))
    for a, X in enumerate((x, y, z)):
        if a in axes:
            m = X > 1.0
            X[m] = 2.0 - X[m]
            sgn[m, a] = -1.0
    rho = 1.2 + 0.3 * np.exp(-((x - 0.3) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2) / 0.02)
    u = 0.3 * np.sin(np.pi * x) * (1 + 0.2 * y) * sgn[:, 0]
    v = 0.2 * np.cos(2 * y + z) * (1 + 0.1 * x) * sgn[:, 1]
    w = 0.15 * np.sin(3 * z + x) * sgn[:, 2]
    p = 1.0 + 0.4 * np.exp(-((x - 0.6) ** 2 + (y - 0.3) ** 2 + (z - 0.4) ** 2) / 0.03)
    g = num.gamma
    cv0 = np.stack([rho, rho * u, rho * v, rho * w, p / (g - 1) + 0.5 * rho * (u * u + v * v + w * w)], axis=1)
    num.dt_imposed = 1e-3
    return Case("mirror_box", mesh["xyz"], mesh["c2v"], patches, num, cv0)


def sod(nx=400, ny=4, nz=4, num=None):
    """Sod shock tube on [0,1]x[0,0.01]^2 hexes: (1,0,1) for x<0.5 and
    (0.125,0,0.1) beyond, slip walls in y/z, supersonic (extrapolation)
    outflow at both x ends, first-order Roe, run to t = 0.2 at CFL 0.5."""
    mesh = meshgen.hex_box(nx, ny, nz, hi=(1.0, 0.01, 0.01))
    if num is None:
        num = Numerics(space_order=1, space_discr=DISCR_ROE, reconst=RECONST_NONE, cfl=0.5)
    out = {"bc_type": BC_OUTFLOW, "outflow_type": 0, "order": 1}
    patches = _patches(mesh, [out, out, SLIP, SLIP, SLIP, SLIP])
    xc = meshgen.cell_centers(mesh)[:, 0]
    left = xc < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    z = np.zeros_like(rho)
    cv0 = conserved(rho, z, z, z, p, num.gamma)
    # imposed first step = the CFL step of the initial state (cubic cells of
    # side h, still gas, sound speed sqrt(gamma) on the left: dt = h/(6c)),
    # so the reference's first-step TIMESTEP rule does not change the run
    h = 1.0 / nx
    num.dt_imposed = num.cfl * h / (6.0 * math.sqrt(num.gamma))
    return Case("sod", mesh["xyz"], mesh["c2v"], patches, num, cv0, end_time=0.2)


def blast_tets(n=64, num=None, seed=0, p_in=100.0, radius=0.1):
    """Spherical blast on n^3 hexes split into 6 jittered tetrahedra (+-0.2h,
    seed 0): rho=1, u=0, p=p_in inside r<radius about the centre, p=1 outside;
    slip walls on all six sides; 2nd-order LSQ, Venkatakrishnan, HLLC, CFL 0.4."""
    mesh = meshgen.tet_box(n, jitter=0.2, seed=seed)
    if num is None:
        num = Numerics(space_order=2, space_discr=DISCR_HLLC, reconst=RECONST_VENKAT, cfl=0.4)
    patches = _patches(mesh, [dict(SLIP, order=2)] * 6)
    c = meshgen.cell_centers(mesh) - 0.5
    r = np.sqrt((c * c).sum(axis=1))
    p = np.where(r < radius, p_in, 1.0)
    rho = np.ones_like(p)
    z = np.zeros_like(p)
    cv0 = conserved(rho, z, z, z, p, num.gamma)
    num.dt_imposed = 1.0  # replaced by the CFL step at t=0 (see first_dt)
    return Case("blast_tets", mesh["xyz"], mesh["c2v"], patches, num, cv0, n_steps=100)


def shock_sphere(n=128, num=None, discr=DISCR_HLLC):
    """Mach-2 planar shock at x=0.2 moving +x into rho=1, p=1, u=0 (gamma 1.4),
    Rankine-Hugoniot post-shock state behind it, density-3 sphere of radius
    0.15 at the centre; n^3 hexes on [0,1]^3; supersonic outflow on the x
    faces (2nd-order patches), slip walls elsewhere; BJ limiter."""
    mesh = meshgen.hex_box(n, n, n)
    if num is None:
        num = Numerics(space_order=2, space_discr=discr, reconst=RECONST_BJ, cfl=0.4)
    out = {"bc_type": BC_OUTFLOW, "outflow_type": 0, "order": 2}
    patches = _patches(mesh, [out, out] + [dict(SLIP, order=2)] * 4)
    c = meshgen.cell_centers(mesh)
    g = num.gamma
    m = 2.0
    rho2 = (g + 1) * m * m / ((g - 1) * m * m + 2)
    p2 = 1.0 + 2 * g / (g + 1) * (m * m - 1)
    u2 = m * math.sqrt(g) * (1.0 - 1.0 / rho2)
    behind = c[:, 0] < 0.2
    d = c - 0.5
    sphere = (d * d).sum(axis=1) < 0.15 ** 2
    rho = np.where(behind, rho2, np.where(sphere, 3.0, 1.0))
    p = np.where(behind, p2, 1.0)
    u = np.where(behind, u2, 0.0)
    z = np.zeros_like(rho)
    cv0 = conserved(rho, u, z, z, p, g)
    num.dt_imposed = 1.0
    return Case("shock_sphere", mesh["xyz"], mesh["c2v"], patches, num, cv0, n_steps=500,
                extra={"rho2": rho2, "p2": p2, "u2": u2})


def adjoint_tets(n=32, num=None, seed=0, pert_seed=1, limiter=RECONST_VENKAT):
    """Uniform Mach-0.5 flow along x (rho=1, p=1/gamma, u=0.5) with a seeded
    +-5% Gaussian perturbation (seed 1) on every conserved variable, on n^3
    hexes split into 6 jittered tetrahedra; second-order Roe.  x-low:
    supersonic-type extrapolation outflow, x-high: subsonic outflow at
    p=1/gamma, slip walls elsewhere, all patches second order."""
    mesh = meshgen.tet_box(n, jitter=0.2, seed=seed)
    if num is None:
        num = Numerics(space_order=2, space_discr=DISCR_ROE, reconst=limiter, cfl=0.4)
    g = num.gamma
    patches = _patches(mesh, [{"bc_type": BC_OUTFLOW, "outflow_type": 0, "order": 2},
                              {"bc_type": BC_OUTFLOW, "outflow_type": 1, "p_out": 1.0 / g, "order": 2}]
                       + [dict(SLIP, order=2)] * 4)
    nc = mesh["c2v"].shape[0]
    one = np.ones(nc)
    cv0 = conserved(one, 0.5 * one, 0 * one, 0 * one, one / g, g)
    rng = np.random.Generator(np.random.PCG64(pert_seed))
    cv0 = cv0 * (1.0 + 0.05 * rng.standard_normal(cv0.shape))
    # keep the y/z momentum perturbations (their mean is zero) relative to |u|
    cv0[:, 2] = 0.05 * rng.standard_normal(nc) * 0.5
    cv0[:, 3] = 0.05 * rng.standard_normal(nc) * 0.5
    num.dt_imposed = 1.0
    return Case("adjoint_tets", mesh["xyz"], mesh["c2v"], patches, num, cv0)


def blast_hex(n=64, num=None, p_in=10.0, radius=0.15):
    """Spherical blast on n^3 hexes: rho=1, p=p_in for r<radius, p=1 outside,
    slip walls, HLLC, BJ limiter (time-unrolled adjoint case)."""
    mesh = meshgen.hex_box(n, n, n)
    if num is None:
        num = Numerics(space_order=2, space_discr=DISCR_HLLC, reconst=RECONST_BJ, cfl=0.4)
    patches = _patches(mesh, [dict(SLIP, order=2)] * 6)
    c = meshgen.cell_centers(mesh) - 0.5
    r = np.sqrt((c * c).sum(axis=1))
    p = np.where(r < radius, p_in, 1.0)
    one = np.ones_like(p)
    z = np.zeros_like(p)
    cv0 = conserved(one, z, z, z, p, num.gamma)
    num.dt_imposed = 1.0
    return Case("blast_hex", mesh["xyz"], mesh["c2v"], patches, num, cv0, n_steps=200)


def open_channel(n=8, num=None, inflow=BC_INFLOW_TOTANG, inflow_type=BCOPT_SUBSONIC, order=2, mach=0.3,
                 seed=3, pert=0.02, injection=0.05, tets=False):
    """A box open to the outside on every side type the path carries: n x
    n/2 x n/2 hexes (or 6 jittered tetrahedra per hex) on [0,1] x [0,0.5]^2,
    uniform Mach-`mach` flow along x (rho = 1, p = 1/gamma, so c = 1 and,
    with cp = 3.5, R = 1) with a seeded +-`pert` perturbation.  x-low: inflow
    (TOTANG: the flow's total pressure and temperature, zero angles; VELTEMP:
    its velocity, temperature and pressure) of the given BCOPT type; x-high:
    subsonic outflow at the static pressure; y faces: farfield at the flow's
    Mach number, pressure and temperature; z-low: injection of
    `injection` mass flux at the flow's temperature (0: a non-burning
    injection wall); z-high: no-slip wall."""
    ny = max(n // 2, 2)
    if tets:
        mesh = meshgen.tet_box(n, jitter=0.2, seed=0)
    else:
        mesh = meshgen.hex_box(n, ny, ny, hi=(1.0, 0.5, 0.5))
    if num is None:
        num = Numerics(space_order=order, space_discr=DISCR_HLLC, reconst=RECONST_BJ, cfl=0.4)
    g = num.gamma
    rgas = num.cp - num.cp / g
    p0, rho0 = 1.0 / g, 1.0
    t0 = p0 / (rho0 * rgas)
    u0 = mach * math.sqrt(g * p0 / rho0)
    fac = 1.0 + 0.5 * (g - 1.0) * mach * mach
    if inflow == BC_INFLOW_TOTANG:
        inl = {"bc_type": inflow, "vals": (p0 * fac ** (g / (g - 1.0)), t0 * fac, 0.0, 0.0, mach),
               "switches": (inflow_type, 0)}
    else:
        inl = {"bc_type": inflow, "vals": (u0, 0.0, 0.0, t0, p0), "switches": (inflow_type, 0)}
    out = {"bc_type": BC_OUTFLOW, "outflow_type": BCOPT_SUBSONIC, "p_out": p0}
    far = {"bc_type": BC_FARFIELD, "vals": (mach, 0.0, 0.0, p0, t0), "switches": (0, 0)}
    inj = {"bc_type": BC_INJECTION, "vals": (injection, t0)}
    wall = {"bc_type": BC_NOSLIPWALL_HFLUX}
    kinds = [inl, out, far, far, inj, wall]
    patches = _patches(mesh, [dict(k, order=min(order, num.space_order)) for k in kinds])
    nc = mesh["c2v"].shape[0]
    one = np.ones(nc)
    cv0 = conserved(rho0 * one, u0 * one, 0 * one, 0 * one, p0 * one, g)
    rng = np.random.Generator(np.random.PCG64(seed))
    cv0 = cv0 * (1.0 + pert * rng.standard_normal(cv0.shape))
    cv0[:, 2] = pert * u0 * rng.standard_normal(nc)
    cv0[:, 3] = pert * u0 * rng.standard_normal(nc)
    num.dt_imposed = 1.0e-3
    return Case("open_channel", mesh["xyz"], mesh["c2v"], patches, num, cv0, n_steps=20)
