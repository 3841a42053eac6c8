"""The reference's limiter-frame sector goldens (sector_limiter_frame_np2.json,
written by make_sector_limiter_frame.py) as cases of this package, for the
oracle's and the device's comparisons with them.

The runs: a 90-degree annulus sector about z (r from 2 mm to 12 mm, 16
cells around, square-graded rings, two z layers), a cylindrical gas jump
at r = 6 mm at rest (utilities/init/RFLU_InitFlowHardCode.F90:839-905,
case "cylds": the post-shock state inside, ambient outside), HLLC, Wray
RK3, eigen-frame Barth-Jespersen (RECONST 10), to t = 4e-6 s; theta0-3.7
is the same sector turned by 3.7 degrees.  The reference's patches: the two planes as a
rotational periodic pair, an NSCBC outflow at r_out, a slip wall at r_in,
the z planes as a translational periodic pair.  Here:

* the planes and the z planes are symmetry (mirror) patches.  The flow is
  axisymmetric and z-invariant, and the mesh is symmetric about the
  sector's bisector (uniform angular spacing) and about each z layer's
  mid-plane, so a cell's image across a plane by reflection is, in position
  and state, its image by the rotation (or translation) of the periodic
  pair;
* r_out is an outflow patch of the .bc's TYPE without the characteristic
  (NSCBC) treatment: no wave reaches r_out by t = 4e-6 (the tests check
  that the outer ring keeps its initial state), so the boundary flux is the
  ambient pressure's either way.

The golden lists each region's cells in its own order; its per-cell values
are compared with the run's as sorted sets of each field (the flow depends
on r only, so each ring's 32 cells share their values)."""
import json
import os

import numpy as np

from rocflu_gb300 import cases, meshgen, refio

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sector_limiter_frame_np2.json")
RUNS = ["theta0-0", "theta0-3.7"]
NAMES = ["q1", "q2", "q3", "q4", "q5"]
MIRRORED = ("plane1", "plane2", "zlow", "zhigh")


def load():
    with open(FIXTURE) as f:
        return json.load(f)


def case(run, reconst=None):
    """(Case, golden cells (n, 5), cell radii) of one run; reconst overrides
    the deck's limiter."""
    g = load()[run]
    grid = {"xyz": np.array(g["grid"]["xyz"]), "hex2v": np.array(g["grid"]["hex2v"], dtype=np.int32),
            "tet2v": np.zeros((0, 4), np.int32), "pri2v": np.zeros((0, 6), np.int32),
            "pyr2v": np.zeros((0, 5), np.int32),
            "patches": [{"name": p["name"], "tris": np.zeros((0, 3), np.int32),
                         "quads": np.array(p["quads"], dtype=np.int32)} for p in g["grid"]["patches"]]}
    num = cases.Numerics(**g["deck"]["numerics"])
    if reconst is not None:
        num.reconst = reconst
    bc = refio.read_deck(g["bc"])
    outer = bc["BC_OUTFLOW"]
    kinds = []
    for p in grid["patches"]:
        if p["name"] in MIRRORED:
            kinds.append({"bc_type": cases.BC_SYMMETRY, "order": 1})
        elif p["name"] == "outer":
            kinds.append({"bc_type": cases.BC_OUTFLOW, "outflow_type": int(float(outer["TYPE"])),
                          "order": int(float(outer["ORDER"]))})
        elif p["name"] == "inner":
            kinds.append({"bc_type": cases.BC_SLIPWALL, "order": g["deck"]["order_bf"]})
        else:
            raise ValueError("unexpected patch %s" % p["name"])
    c = refio.case_from_centaur(grid, kinds, num, name="sector_limiter_frame_" + run)
    ini = g["deck"]["initflow"]
    cc = meshgen.cell_centers({"xyz": c.xyz, "c2v": c.c2v})
    r = np.hypot(cc[:, 0], cc[:, 1])
    inside = r < ini["RVAL1"]
    rho = np.where(inside, ini["RVAL2"], ini["RVAL5"])
    p = np.where(inside, ini["RVAL4"], ini["RVAL6"])
    z = np.zeros_like(r)  # RVAL3 = 0: at rest
    assert ini["RVAL3"] == 0.0
    c.cv0 = cases.conserved(rho, z, z, z, p, num.gamma)
    c.end_time = g["deck"]["end_time"]
    gold = np.concatenate([np.stack([np.array(g["gas"][k][n]) for n in NAMES], axis=1)
                           for k in sorted(g["gas"])])
    return c, gold, r


def sorted_distance(cv, gold):
    """Per field, the largest difference of the sorted cell values over the
    field's largest golden magnitude; the three momenta share one scale."""
    mom = np.abs(gold[:, 1:4]).max()
    scales = [np.abs(gold[:, 0]).max(), mom, mom, mom, np.abs(gold[:, 4]).max()]
    return np.array([np.abs(np.sort(cv[:, k]) - np.sort(gold[:, k])).max() / scales[k] for k in range(5)])
