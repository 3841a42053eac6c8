"""The reference's file formats (rocflu_gb300/refio.py): fluid dumps against
the reference harness's own reader, CENTAUR ASCII grids by round trip, and
a reference-format grid through the solver against the reference's golden."""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from rocflu_gb300 import cases, meshgen, refio

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_fluid_dump_matches_reference_reader(tmp_path):
    """The writer reproduces, byte for byte, the dump whose parse by the
    reference harness's read_fluid_dump is stored in the fixture
    (tests/golden/make_fluid_dump_fixture.py), and the reader returns the
    same values."""
    fx = json.load(open(os.path.join(GOLDEN, "fluid_dump_v5.json")))
    ref = fx["reference_reader"]
    cv = np.array(ref["cv"]).T
    nscbc = {int(k): np.array(v).T for k, v in ref["nscbc"].items()}
    path = refio.fluid_dump_name(str(tmp_path), ref["step"], ref["region"])
    assert os.path.basename(path) == fx["name"]
    refio.write_fluid_dump(path, cv, ref["step"], ref["time"], ref["region"], nscbc=nscbc)
    assert open(path, "rb").read() == bytes.fromhex(fx["bytes_hex"])
    assert not os.path.exists(path + ".tmp")
    d = refio.read_fluid_dump(path)
    assert (d["step"], d["time"], d["region"], d["form"]) == (ref["step"], ref["time"], ref["region"], ref["form"])
    np.testing.assert_array_equal(d["cv"], cv)
    assert list(d["nscbc"]) == [2]
    np.testing.assert_array_equal(d["nscbc"][2], nscbc[2])


@pytest.mark.parametrize("wide", [True, False])
@pytest.mark.parametrize("kind", ["hex", "tets"])
def test_centaur_ascii_round_trip(tmp_path, kind, wide):
    mesh = meshgen.hex_box(3, 2, 4) if kind == "hex" else meshgen.tet_box(3, jitter=0.2, seed=0)
    key = "hex2v" if kind == "hex" else "tet2v"
    patches = []
    for k, p in enumerate(mesh["patches"]):
        bf = p["bf2v"]
        tri = bf[:, 3] < 0
        patches.append({"bc_type": 10 + k, "name": p["name"], "tris": bf[tri, :3], "quads": bf[~tri]})
    path = str(tmp_path / "box.hyb.asc")
    refio.write_centaur_ascii(path, mesh["xyz"], {key: mesh["c2v"]}, patches, title="round trip", wide=wide)
    g = refio.read_centaur_ascii(path)
    assert g["title"] == "round trip"
    tol = 0.0 if wide else 1e-9
    np.testing.assert_allclose(g["xyz"], mesh["xyz"], rtol=tol, atol=tol)
    np.testing.assert_array_equal(g[key], mesh["c2v"])
    for other, _ in refio.CELL_BLOCKS:
        if other != key:
            assert g[other].shape[0] == 0
    assert [p["bc_type"] for p in g["patches"]] == [p["bc_type"] for p in patches]
    for a, b in zip(g["patches"], patches):
        assert a["name"] == b["name"]
        np.testing.assert_array_equal(a["tris"], b["tris"])
        np.testing.assert_array_equal(a["quads"], b["quads"])


def test_gas_jump_from_centaur_grid_matches_reference_golden(tmp_path):
    """The closed gas-jump box written as a CENTAUR ASCII grid, read back and
    run (HLLC, WENO-XYZ, first-order slip walls, Wray RK3 to t = 1.05e-4)
    reaches the reference's golden within the harness's 1e-10; its final
    state written as a fluid dump reads back unchanged."""
    from golden import gas_jump

    golden, layers, scales = gas_jump.load()
    ref = cases.gas_jump_closed()
    mesh = {"xyz": ref.xyz, "c2v": ref.c2v}
    patches = [{"bc_type": 5, "name": p.name, "tris": np.zeros((0, 3), int), "quads": p.bf2v} for p in ref.patches]
    path = str(tmp_path / "rectshktb.hyb.asc")
    refio.write_centaur_ascii(path, mesh["xyz"], {"hex2v": mesh["c2v"]}, patches, title="rectshktb")
    g = refio.read_centaur_ascii(path)
    c = refio.case_from_centaur(g, [dict(cases.SLIP, order=1)] * len(g["patches"]), ref.num, ref.cv0)
    o = Oracle(c)
    o.run(100000, 0.0, ref.end_time)
    cv, _ = o.state()
    err = np.abs(cv - layers[gas_jump.layer_of_cells(c)]) / scales
    assert err.max() <= 1e-10, err.max(axis=0)
    dump = refio.fluid_dump_name(str(tmp_path), 569, 1)
    refio.write_fluid_dump(dump, cv, 569, golden["time"], 1)
    np.testing.assert_array_equal(refio.read_fluid_dump(dump)["cv"], cv)


def test_gas_jump_case_is_what_the_reference_deck_states():
    """cases.gas_jump_closed() carries the numerics, end time and patch
    conditions that the reference's test deck (with the golden's overrides)
    and boundary file state, as refio read them when the fixture was made."""
    import dataclasses

    fx = json.load(open(os.path.join(GOLDEN, "gas_jump_closed_creconst0_np2.json")))["deck"]
    c = cases.gas_jump_closed()
    num = dataclasses.asdict(c.num)
    assert {k: num[k] for k in fx["numerics"]} == fx["numerics"]
    assert num["c_reconst"] == 0  # the golden's override CRECONSTC 0
    assert c.end_time == fx["end_time"]
    assert [{"bc_type": p.bc_type, "order": p.order} for p in c.patches] == fx["patch_kinds"]


def test_deck_and_bc_syntax():
    deck = refio.read_deck("""# NUMERICS
CFL      0.4	! CFL number
DISCR    3      ! HLLC
ORDER    2
RECONST  11
#
# TIMESTEP
FLOWTYPE   1
MAXTIME    2.0E-04
TIMESTEP   1.0E-09
DTMINLIMIT 2.0E-10
RKSCHEME   2
#
# REFERENCE
GAMMA   1.4
CP      1004.64
#
""")
    num, end_time, order_bf = refio.numerics_from_deck(deck)
    assert (num.cfl, num.space_discr, num.space_order, num.reconst, num.rk_scheme) == (0.4, 3, 2, 11, 2)
    assert (end_time, num.dt_imposed, num.dt_min_limit, order_bf) == (2.0e-4, 1.0e-9, 2.0e-10, 1)
    bc = refio.read_deck("""# BC_SLIPW
PATCH      3 6
NAME       Walls
#

# BC_OUTFLOW
PATCH      1 2
TYPE       1
PRESS      82700.0
ORDER      2
#

# END
""")
    kinds = refio.patch_kinds_from_bc(bc, 6)
    assert kinds[0] == kinds[1] == {"bc_type": cases.BC_OUTFLOW, "outflow_type": 1, "p_out": 82700.0, "order": 2}
    assert all(k == {"bc_type": cases.BC_SLIPWALL, "order": 1} for k in kinds[2:])
    num1, _, _ = refio.numerics_from_deck(refio.apply_overrides(deck, {"NUMERICS/CRECONSTC": 1}))
    assert num1.c_reconst == 1 and num1.c_reconst_weight == 1.0
    with pytest.raises(ValueError):
        refio.numerics_from_deck(refio.apply_overrides(deck, {"NUMERICS/CRECONSTC": 2}))
    with pytest.raises(ValueError, match="RELPATCH"):
        refio.patch_kinds_from_bc(refio.read_deck("# BC_PERIODIC\nPATCH 1 6\n#\n"), 6)


def test_bc_sections_of_the_open_patches():
    """Inflow, farfield, injection and no-slip sections in the .bc syntax of
    modflu/RFLU_ModReadBcInputFile.F90: keys to BCDAT / BCSWI order, angles
    in degrees converted with the reference's deg2rad, MACH and PRESS only
    read for a non-subsonic inflow."""
    import math

    bc = refio.read_deck("""
# BC_INFLOW_VELTEMP
PATCH       1 1
TYPE        1   ! subsonic: PRESS not needed
TEMP        348.29
VELX        138.92
VELY        0.0
VELZ        0.0
ORDER       2
#
# BC_FARF
PATCH      2 2
MACH       0.5
ATTACK     90.0
SLIP       0.0
PRESS      1.0E+05
TEMP       300.0
#
# BC_INFLOW
PATCH      3 3
TYPE       0
PTOT       2.0E+05
TTOT       400.0
BETAH      30.0
BETAV      0.0
MACH       1.5
#
# BC_INJECT
PATCH      4 4
MFRATE     2.0
TEMP       2500.0
#
# BC_NOSLIP
PATCH      5 5
#
# BC_NOSLIP_TEMP
PATCH      6 6
TEMP       300.0
#
# END
""")
    k = refio.patch_kinds_from_bc(bc, 6)
    assert k[0] == {"bc_type": cases.BC_INFLOW_VELTEMP, "switches": (1, 0), "vals": (138.92, 0.0, 0.0, 348.29, 0.0),
                    "order": 2}
    assert k[1]["bc_type"] == cases.BC_FARFIELD and k[1]["switches"] == (0, 0)
    assert abs(k[1]["vals"][1] - math.pi / 2) <= 1e-15 and k[1]["vals"][3:] == (1.0e5, 300.0)
    assert k[2]["bc_type"] == cases.BC_INFLOW_TOTANG and k[2]["switches"] == (0, 0)
    assert abs(k[2]["vals"][2] - math.pi / 6) <= 1e-15 and k[2]["vals"][4] == 1.5
    assert k[3] == {"bc_type": cases.BC_INJECTION, "vals": (2.0, 2500.0), "order": 1}
    assert k[4]["bc_type"] == cases.BC_NOSLIPWALL_HFLUX and k[5]["bc_type"] == cases.BC_NOSLIPWALL_TEMP
