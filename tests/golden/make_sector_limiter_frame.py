"""Writes tests/golden/sector_limiter_frame_np2.json from the reference's own
goldens of the limiter-frame sector runs (its tests/goldens/sector/
limiter-frame/theta0-0/np2 and theta0-3.7/np2 golden.json: the state the
Fortran solver reached at t = 4e-6 on two ranks with the eigen-frame
Barth-Jespersen limiter, RECONST 10, conserved variables per region in the
region's cell order), keeping per run the specification, the time, the
per-region fields and the totals, plus:

* the grid, as the reference's own mesh tool writes it for that
  specification (utilities/mesh/sector_mesh.py, run here with the
  arguments the reference's test harness passes it,
  tests/rocpicl_tests/case.py: SectorGrid.write), read back from its
  CENTAUR file by rocflu_gb300.refio: vertices, hexahedra, patches;
* the .bc file the tool writes beside it (the patches' conditions);
* the numerics and the initial-flow values of the reference's test deck
  (tests/templates/rectshktb.inp with the run's overrides).

Run once where the reference source tree is present:

    python tests/golden/make_sector_limiter_frame.py <reference source tree>
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rocflu_gb300 import refio  # noqa: E402

RUNS = ["theta0-0", "theta0-3.7"]
SRC = os.path.join("tests", "goldens", "sector", "limiter-frame", "%s", "np2", "golden.json")
TOOL = os.path.join("utilities", "mesh", "sector_mesh.py")
DECK = os.path.join("tests", "templates", "rectshktb.inp")
INIT_KEYS = ["RVAL1", "RVAL2", "RVAL3", "RVAL4", "RVAL5", "RVAL6"]


def grid_of(ref_root, g):
    """The reference tool's mesh for a golden's grid specification."""
    args = ["cylds", "--angle", repr(g["angle"]), "--theta0", repr(g["theta0"]), "--r-out", repr(g["r_out"]),
            "--ntheta", str(g["ntheta"]), "--z", repr(g["z"][0]), repr(g["z"][1]), "--nz", str(g["nz"])]
    if g.get("r_in") is None or g.get("core") is not None or g.get("max_cell") or g.get("full"):
        raise SystemExit("only the annulus layout without refinement rings is extracted")
    args += ["--r-in", repr(g["r_in"])]
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([sys.executable, os.path.join(ref_root, TOOL)] + args, cwd=d, check=True,
                       capture_output=True)
        grid = refio.read_centaur_ascii(os.path.join(d, "cylds.hyb.asc"))
        with open(os.path.join(d, "cylds.bc")) as f:
            bc = f.read()
    return {"xyz": grid["xyz"].tolist(), "hex2v": grid["hex2v"].tolist(),
            "patches": [{"name": p["name"], "quads": p["quads"].tolist()} for p in grid["patches"]]}, bc


def main(ref_root):
    with open(os.path.join(ref_root, DECK)) as f:
        template = f.read()
    out = {}
    for run in RUNS:
        src = SRC % run
        with open(os.path.join(ref_root, src)) as f:
            g = json.load(f)
        grid, bc = grid_of(ref_root, g["spec"]["grid"])
        deck = refio.apply_overrides(refio.read_deck(template), g["spec"]["inp"])
        num, end_time, order_bf = refio.numerics_from_deck(deck)
        out[run] = {"source": src, "spec": g["spec"], "time": g["state"]["time"], "gas": g["state"]["gas"],
                    "totals": g["state"]["totals"], "grid": grid, "bc": bc,
                    "deck": {"numerics": num.__dict__, "end_time": end_time, "order_bf": order_bf,
                             "initflow": {k: float(deck["INITFLOW"][k]) for k in INIT_KEYS}}}
    dst = os.path.join(HERE, "sector_limiter_frame_np2.json")
    with open(dst, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference source tree>" % sys.argv[0])
    main(sys.argv[1])
