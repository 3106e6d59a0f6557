"""The vectorised A-A step kernel (V cells per thread, 4- to 16-byte population
vectors, lbm_vec.cuh) against the one-cell-per-lane kernel on the same
geometries: odd and even steps, with and without averaging, every storage it
serves and both block widths.  The two kernels run the same float32 collision
(src/engine.js:277-319 rearranged as in collide_fast); they may contract a
multiply-add differently, so populations agree to float32 rounding (one unit of
the stored deviation for the 16-bit formats) rather than bit for bit."""
import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E

pytestmark = pytest.mark.gpu

RUN = dict(K=3.0, aniso=10.0, u=0.06, tau=0.51, steps=200, avg=50, every=50)
SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})
CASES = {"small_baffle": ag.AirboxSpec(**SMALL), "config1": ag.config1_spec(), "yaw_seed3": ag.random_spec(3, dx=4.0),
         "fine_yaw": ag.random_spec(11, dx=2.5)}
TOL = {"f32": 1e-6, "f16": 1.3e-4, "bf16": 1e-3}
_GEOMS = {}


def geom(name):
    if name not in _GEOMS:
        spec = CASES[name]
        _GEOMS[name] = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
    return _GEOMS[name]


def run(g, storage, steps_plain, steps_acc):
    S = E.Simulation(g, {**RUN, "storage": storage, "allowBf16": True})
    S.step(steps_plain)
    S.step(steps_acc, True)
    info = S.refresh()
    return S.get_f(), S.get_acc(), info


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("storage,V", [("f32", 2), ("f32", 4), ("f16", 2), ("f16", 4), ("bf16", 4)])
def test_vec_kernel_matches_one_cell_kernel(name, storage, V, monkeypatch):
    g = geom(name)
    monkeypatch.setenv("ABX_VEC", "1")
    monkeypatch.setenv("ABX_VEC_V", str(V))
    f, acc, info = run(g, storage, 7, 6)
    assert info.vec_width == V
    assert 0 < info.vec_interior_cells <= g.nf
    monkeypatch.setenv("ABX_VEC", "0")
    f0, acc0, info0 = run(g, storage, 7, 6)
    assert info0.vec_width == 0
    assert np.all(np.isfinite(f))
    assert np.abs(f - f0).max() < TOL[storage]
    assert np.abs(acc - acc0).max() < 1e-5


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_vec_kernel_full_run_kpis(storage, monkeypatch):
    """A whole 6000/2000 solve of config1 through the vectorised kernel keeps every KPI within 0.5 % of the
    one-cell-per-lane kernel's solve."""
    g = geom("config1")
    run6 = dict(RUN, steps=6000, avg=2000, every=150)
    out = {}
    for vec in ("1", "0"):
        monkeypatch.setenv("ABX_VEC", vec)
        S = E.Simulation(g, {**run6, "storage": storage})
        S.run()
        out[vec] = S.evaluate()["metrics"]
    for k in ("gamma", "gammaCore", "maxToMean", "zeta"):
        assert out["1"][k] == pytest.approx(out["0"][k], rel=5e-3), k
