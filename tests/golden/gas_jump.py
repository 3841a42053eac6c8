"""The reference's closed gas-jump golden (gas_jump_closed_creconst0_np2.json,
written by make_gas_jump_closed.py) per x layer of its 8^3 box, for the
oracle's and the device's comparisons with it.

The run was split into two regions of four x layers, region 1 the upper half
in x and region 2 the lower, each listed in its own cell order with x
varying fastest; the flow depends on x only (checked here to 1e-12 across y
and z)."""
import json
import os

import numpy as np

NAMES = ["q1", "q2", "q3", "q4", "q5"]


def load():
    """(golden dict, (8, 5) layer values, (5,) comparison scales): a field's
    maximum magnitude over both regions, the momentum components on one
    scale, as the reference harness compares them."""
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "gas_jump_closed_creconst0_np2.json")) as f:
        golden = json.load(f)
    layers = np.zeros((8, 5))
    for region, first in (("1", 4), ("2", 0)):
        for k, name in enumerate(NAMES):
            arr = np.array(golden["gas"][region][name]).reshape(-1, 4)
            spread = np.abs(arr - arr[0]).max()
            assert spread <= 1e-12 * max(np.abs(arr).max(), 1.0), (region, name, spread)
            layers[first:first + 4, k] = arr[0]
    allv = {n: [v for r in golden["gas"].values() for v in r[n]] for n in NAMES}
    mom = max(abs(v) for n in ("q2", "q3", "q4") for v in allv[n])
    scales = np.array([max(abs(v) for v in allv["q1"]), mom, mom, mom, max(abs(v) for v in allv["q5"])])
    return golden, layers, scales


def layer_of_cells(case, width=0.001):
    """x layer (0..7) of every cell of the case, from its centroid."""
    from rocflu_gb300 import meshgen

    x = meshgen.cell_centers({"xyz": case.xyz, "c2v": case.c2v})[:, 0]
    return np.floor(x / width).astype(int)
