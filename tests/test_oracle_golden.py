"""The oracle (C restatement of src/engine.js) against fixtures made by running
the reference's own Python CLI (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from oracle import oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "airbox_cfd_golden.npz"))
CASES = ["small_baffle", "wide_low", "fine_cells"]
SPECS = {
    "small_baffle": dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0,
                         dx=5.0, baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21}),
    "wide_low": dict(Lx=201.13, Ly=88.71, Lz=151.37, t=3.07, d_in=55.21, stub=30.41, pleat=40.0,
                     dx=4.0, hole_x=88.33),
    "fine_cells": dict(Lx=96.17, Ly=71.43, Lz=80.29, t=2.93, d_in=30.11, stub=15.37, pleat=30.0,
                       dx=2.5, baffle={"z": 33.71, "x0": 40.13, "x1": 93.24, "y0": 55.07}),
}


def test_parse_stl_binary_matches_reference():
    buf = GOLD["stl_binary"].tobytes()
    assert np.array_equal(O.parse_stl(buf), GOLD["stl_binary_parsed"])


def test_parse_stl_ascii_matches_reference():
    buf = GOLD["stl_ascii"].tobytes()
    assert np.array_equal(O.parse_stl(buf), GOLD["stl_ascii_parsed"])


def test_parse_stl_errors_and_regex_edges():
    with pytest.raises(O.OracleError, match="keine Dreiecke"):
        O.parse_stl(b"solid x\nvertex 1 2 3\nendsolid")
    # a malformed number token becomes NaN, like JS Number("1.2.3")
    t = O.parse_stl(b"vertex 1.2.3 0 0 vertex 1 0 0 vertex 0 1 0")
    assert np.isnan(t[0]) and t[1] == 0 and t[3] == 1
    # a vertex keyword without three numbers is skipped
    t = O.parse_stl(b"vertex 9 9\nvertex 1 2 3\nvertex 4 5 6\nvertex 7 8 9\n")
    assert list(t) == [1, 2, 3, 4, 5, 6, 7, 8, 9]


def test_frame_matches_reference_to_local():
    pts = GOLD["frame_points"]
    n = 0
    for key in GOLD.files:
        if not key.startswith("frame_") or key == "frame_points":
            continue
        _, ds, face = key.split("_")
        dax, dsg = "xyz".index(ds[0]), ds[1]
        seal = float(GOLD[key][0])
        want = GOLD[key][1:].reshape(-1, 3)
        p = {"sealAxis": dax, "sealSign": -1 if dsg == "p" else 1, "seal": seal,
             "inletAxis": "xyz".index(face[0]), "inletSign": -1 if face.endswith("min") else 1,
             "inletYaw": 0, "dx": 1, "pleat": 40}
        fr = O.Frame()
        pp = O.prep_params(p)
        O.lib().ora_make_frame(pp, fr)
        got = np.empty_like(want)
        for r, q in enumerate(pts):
            out = (O.C.c_double * 3)()
            O.lib().ora_to_local(fr, (O.C.c_double * 3)(*q), out)
            got[r] = list(out)
        assert np.array_equal(got, want), key
        n += 1
    assert n == 24


@pytest.mark.parametrize("name", CASES)
def test_voxelizer_and_masks_match_reference(name):
    spec = ag.AirboxSpec(**SPECS[name])
    tris = ag.build_airbox(spec)
    g = O.prepare(tris, spec.prepare_params(), keep_fine=True)
    shape = tuple(GOLD[f"vox_{name}_shape"])
    assert (g.g.nxf, g.g.nyf, g.g.nzf) == shape
    nfine = int(np.prod(shape))
    fine = np.unpackbits(GOLD[f"vox_{name}_fine"])[:nfine]
    assert np.array_equal(g.fine(), fine), "fine voxel grid differs from airbox_cfd.voxelize"
    cshape = tuple(GOLD[f"vox_{name}_coarse_shape"])
    assert (g.nx, g.ny, g.nz) == cshape
    n = int(np.prod(cshape))
    assert np.array_equal(g.solid(), np.unpackbits(GOLD[f"vox_{name}_solid"])[:n])
    assert np.array_equal(g.fluid(), np.unpackbits(GOLD[f"vox_{name}_fluid"])[:n])


@pytest.mark.parametrize("name", ["small_baffle", "wide_low"])
def test_evaluate_formulas_match_reference_report(name):
    """report() of the reference's Python CLI (airbox_cfd.py:296-314) on its own averaged fields of a 60-step run
    against the oracle's evaluate() (src/engine.js:632-660) on the same fields: the KPI formulas agree.  The CLI
    sums float32 arrays with numpy's pairwise float32 sums where engine.js sums in float64, hence the tolerance."""
    spec = ag.AirboxSpec(**SPECS[name])
    g = O.prepare(ag.build_airbox(spec), spec.prepare_params())
    S = O.OracleSim(g, dict(K=3.0, aniso=10.0, u=0.06, tau=0.51))
    cells = S.cells()
    acc = np.concatenate([GOLD[f"report_{name}_{k}"].ravel()[cells] for k in ("ux", "uy", "uz", "rho")])
    m, _ = S.evaluate(acc.astype(np.float32))
    ref = dict(zip(("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean", "zeta"),
                   GOLD[f"report_{name}_kpi"]))
    for k in ("gamma", "gammaCore", "maxToMean", "zeta"):
        assert abs(m[k] - ref[k]) <= 2e-5 * abs(ref[k]), (k, m[k], ref[k])
    # shares of cells: counts over the core (cn cells) and the layer (n cells) agree to one cell
    for k, n in (("lowCore", m["cn"]), ("highCore", m["cn"]), ("reverse", m["n"])):
        assert abs(m[k] - ref[k]) * n <= 1 + 1e-9, (k, m[k], ref[k])
    assert 0 < ref["lowCore"] < 1 and ref["zeta"] != 0
