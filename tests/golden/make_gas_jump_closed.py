"""Writes tests/golden/gas_jump_closed_creconst0_np2.json from the reference's
own golden of the closed gas-jump box (its tests/goldens/box/gas-jump/
closed-creconst0/np2/golden.json: the state the Fortran solver reached at
t = 1.05e-4 on two ranks, conserved variables per region in the region's
cell order), keeping the run specification, the time, the per-region fields
and the totals.  Run once where the reference source tree is present:

    python tests/golden/make_gas_jump_closed.py /root/reference
"""
import json
import os
import sys

SRC = os.path.join("tests", "goldens", "box", "gas-jump", "closed-creconst0", "np2", "golden.json")


def main(ref_root):
    with open(os.path.join(ref_root, SRC)) as f:
        g = json.load(f)
    out = {"source": SRC, "spec": g["spec"], "time": g["state"]["time"],
           "gas": g["state"]["gas"], "totals": g["state"]["totals"]}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gas_jump_closed_creconst0_np2.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
