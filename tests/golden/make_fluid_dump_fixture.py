"""Writes tests/golden/fluid_dump_v5.json: the bytes of a fluid dump written by
rocflu_gb300.refio.write_fluid_dump (7 cells, 5 variables, one NSCBC patch of
2 faces) and what the reference test harness's own reader
(tests/rocpicl_tests/outputs.py: read_fluid_dump, in the reference source
tree) returns for them, so that the writer's format is checked against the
reference's reader without that tree.  Run once where it is present:

    python tests/golden/make_fluid_dump_fixture.py /root/reference
"""
import importlib.util
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from rocflu_gb300 import refio  # noqa: E402


def sample():
    rng = np.random.default_rng(11)
    cv = rng.standard_normal((7, 5))
    return {"cv": cv, "step": 1234, "time": 1.05e-4, "region": 3, "nscbc": {2: rng.standard_normal((2, 5))}}


def main(ref_root):
    spec = importlib.util.spec_from_file_location(
        "ref_outputs", os.path.join(ref_root, "tests", "rocpicl_tests", "outputs.py"))
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    s = sample()
    with tempfile.TemporaryDirectory() as d:
        path = refio.fluid_dump_name(d, s["step"], s["region"])
        refio.write_fluid_dump(path, s["cv"], s["step"], s["time"], s["region"], nscbc=s["nscbc"])
        raw = open(path, "rb").read()
        r = ref.read_fluid_dump(path)
    parsed = {"step": r["step"], "time": r["time"], "region": r["region"], "form": r["form"],
              "cv": [list(a) for a in r["cv"]], "nscbc": {str(k): [list(a) for a in v] for k, v in r["nscbc"].items()}}
    assert np.array_equal(np.array(parsed["cv"]).T, s["cv"])
    out = {"name": os.path.basename(path), "bytes_hex": raw.hex(), "reference_reader": parsed}
    with open(os.path.join(HERE, "fluid_dump_v5.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", os.path.join(HERE, "fluid_dump_v5.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python %s <reference source tree>" % sys.argv[0])
    main(sys.argv[1])
