"""Writes tests/golden/gas_jump_symmetry_np1.json from the reference's own
golden of the symmetry gas-jump box (its tests/goldens/box/gas-jump/
symmetry/np1/golden.json: the state the Fortran solver reached at
t = 1.05e-4 on one rank with symmetry patches on all six sides, conserved
variables in the region's cell order, x varying fastest, then y, then z),
keeping the run specification, the time, the field values and the totals.
Run once where the reference source tree is present:

    python tests/golden/make_gas_jump_symmetry.py <reference source tree>
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join("tests", "goldens", "box", "gas-jump", "symmetry", "np1", "golden.json")


def main(ref_root):
    with open(os.path.join(ref_root, SRC)) as f:
        g = json.load(f)
    out = {"source": SRC, "spec": g["spec"], "time": g["state"]["time"], "gas": g["state"]["gas"],
           "totals": g["state"]["totals"]}
    dst = os.path.join(HERE, "gas_jump_symmetry_np1.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference source tree>" % sys.argv[0])
    main(sys.argv[1])
