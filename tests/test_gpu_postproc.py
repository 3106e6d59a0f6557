"""Post-processing of the averages on the GPU against the oracle's
restatement of the reference: field3d (src/engine.js:698-719), the cut
planes of evaluate (:662-680) and the streamlines (:721-758).

Given the same float32 averages the GPU kernels run the reference's float64
arithmetic in its order, so the outputs must be bit-identical: first with the
averages of a cpuStep-exact run (identical to the oracle's own run), then
with the averages a float32 run produced (fed to the oracle), and with a
partial bounce-back field that removes cells from the air.
"""
import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})
RUN = dict(K=3, aniso=10, u=0.06, tau=0.51, steps=300, avg=100, every=50)


def setup(spec=None):
    spec = spec or ag.AirboxSpec(**SMALL)
    tris = ag.build_airbox(spec)
    g = E.prepare({"tris": tris, **spec.prepare_params()})
    og = O.prepare(tris, spec.prepare_params())
    return g, og


def check_all(S, OS, acc, ns=None):
    (spd, pst, loss), kB, pin, rr = OS.field3d(acc, ns)
    v = S.field3d()
    assert v["kB"] == kB and v["_pin"] == pin and v["_rhoRef"] == rr
    sh = spd.shape
    for name, ref in (("spd", spd), ("pst", pst), ("loss", loss)):
        assert np.array_equal(v[name].reshape(sh), ref, equal_nan=True), name
    assert np.isfinite(spd).sum() > 100
    pl, meta = OS.planes(acc, ns)
    got = S.planes()
    assert (got["_ic"], got["_jc"], got["_jlow"]) == meta
    nx, ny, nz = sh
    P, Q = nx * nz, nz * ny
    flat = np.concatenate([got["planInlet"]["speed"], got["planInlet"]["ua"], got["planInlet"]["ub"],
                           got["planLow"]["speed"], got["planLow"]["ua"], got["planLow"]["ub"],
                           got["lon"]["speed"], got["lon"]["ua"], got["lon"]["ub"]])
    assert flat.size == 6 * P + 3 * Q
    assert np.array_equal(flat, pl, equal_nan=True)
    pts, sp, off = OS.streamlines(acc, ns)
    lines = S.streamlines()
    assert len(off) > 5 and off[-1] == len(sp)
    assert np.array_equal(lines["off"], off)
    assert np.array_equal(lines["spd"], sp)
    assert np.array_equal(lines["pts"], pts)


def test_postprocessing_of_exact_run_matches_oracle():
    g, og = setup()
    S = E.Simulation(g, dict(RUN, storage="f32exact"))
    S.run()
    OS = O.OracleSim(og, RUN)
    acc, _ = OS.simulate(RUN["steps"], RUN["avg"], RUN["every"])
    assert np.array_equal(S.get_acc(), acc)          # the averages agree, so must everything after them
    check_all(S, OS, acc)


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_postprocessing_of_fast_runs_matches_oracle_on_their_averages(storage):
    g, og = setup(ag.random_spec(3, dx=4.0))
    S = E.Simulation(g, dict(RUN, storage=storage))
    S.run()
    OS = O.OracleSim(og, RUN)
    check_all(S, OS, S.get_acc())


def test_postprocessing_with_partial_bounce_back():
    g, og = setup()
    OS = O.OracleSim(og, RUN)
    ns = np.zeros(OS.NF, np.float32)
    ns[::7] = 1.0                                     # cells that stop counting as air
    ns[3::11] = 0.4
    S = E.Simulation(g, dict(RUN, storage="f32exact"), ns=ns)
    S.run()
    acc, _ = OS.simulate(RUN["steps"], RUN["avg"], RUN["every"], ns=ns)
    assert np.array_equal(S.get_acc(), acc)
    check_all(S, OS, acc, ns)


def test_evaluate_returns_the_reference_result_object():
    g, _ = setup()
    res = E.simulate(g, dict(RUN, steps=60, avg=20, every=30))
    for k in ("metrics", "hist", "fmap", "planInlet", "planLow", "lon", "vol", "lines", "frame"):
        assert k in res, k
    assert res["vol"]["spd"].size == g.nx * g.ny * g.nz
    assert res["lines"]["off"][0] == 0
