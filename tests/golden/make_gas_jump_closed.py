"""Writes tests/golden/gas_jump_closed_creconst0_np2.json and
tests/golden/gas_jump_closed_np2.json from the reference's own goldens of
the closed gas-jump box (its tests/goldens/box/gas-jump/closed-creconst0/np2
and closed/np2 golden.json, CRECONSTC 0 and 1: the state the Fortran solver
reached at t = 1.05e-4 on two ranks, conserved variables per region in the
region's cell order), keeping the run specification, the time, the
per-region fields and the totals, plus the numerics and patch conditions
that the reference's test deck and boundary file state for that run, as
rocflu_gb300.refio reads them.  Run once where the reference source tree is
present:

    python tests/golden/make_gas_jump_closed.py /root/reference
"""
import dataclasses
import importlib.util
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rocflu_gb300 import refio  # noqa: E402

SRCS = {"gas_jump_closed_creconst0_np2.json": os.path.join("tests", "goldens", "box", "gas-jump", "closed-creconst0",
                                                          "np2", "golden.json"),
        "gas_jump_closed_np2.json": os.path.join("tests", "goldens", "box", "gas-jump", "closed", "np2", "golden.json")}
DECK = os.path.join("tests", "templates", "rectshktb.inp")


def deck_settings(ref_root, spec):
    """The run's numerics and patch conditions as the reference deck states
    them: the test template deck with the golden's overrides, and the
    harness's boundary file for its bc layout (tests/rocpicl_tests/case.py:
    bc_text), read by rocflu_gb300.refio."""
    with open(os.path.join(ref_root, DECK)) as f:
        deck = refio.apply_overrides(refio.read_deck(f.read()), spec["inp"])
    num, end_time, order_bf = refio.numerics_from_deck(deck)
    hspec = importlib.util.spec_from_file_location("ref_case", os.path.join(ref_root, "tests", "rocpicl_tests", "case.py"))
    hcase = importlib.util.module_from_spec(hspec)
    hspec.loader.exec_module(hcase)
    kinds = refio.patch_kinds_from_bc(refio.read_deck(hcase.bc_text(spec["bc"])), 6, order_bf)
    return {"numerics": dataclasses.asdict(num), "end_time": end_time, "patch_kinds": kinds}


def main(ref_root):
    for name, src in SRCS.items():
        with open(os.path.join(ref_root, src)) as f:
            g = json.load(f)
        out = {"source": src, "spec": g["spec"], "time": g["state"]["time"],
               "gas": g["state"]["gas"], "totals": g["state"]["totals"],
               "deck": deck_settings(ref_root, g["spec"])}
        dst = os.path.join(HERE, name)
        with open(dst, "w") as f:
            json.dump(out, f, indent=0)
        print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference source tree>" % sys.argv[0])
    main(sys.argv[1])
