"""Batched variants on the GPU: several airboxes of different size and
parameters advanced by one launch per step must give, variant by variant,
exactly what the same runs give one at a time (the batched kernel runs the
same per-cell arithmetic), with or without the autotuner's shape, and a
variant that goes unstable must stop alone."""
import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import batch as BT
from airboxcalc_gb300 import engine as E

pytestmark = pytest.mark.gpu

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})
RUN = dict(K=3, aniso=10, u=0.06, tau=0.51, steps=120, avg=40, every=30)


def variants():
    specs = [ag.AirboxSpec(**SMALL), ag.random_spec(3, dx=4.0), ag.random_spec(8, dx=5.0)]
    geoms = [E.prepare({"tris": ag.build_airbox(s), **s.prepare_params()}) for s in specs]
    params = [dict(RUN, K=1.5), dict(RUN, K=3.0, u=0.05), dict(RUN, K=6.0, tau=0.52)]
    return geoms, params


def individual(g, p):
    S = E.Simulation(g, p)
    S.run()
    return S.evaluate(), S.get_acc()


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("tuned", [False, True])
def test_batch_matches_individual_runs(storage, tuned):
    geoms, params = variants()
    params = [dict(p, storage=storage, allowBf16=True) for p in params]
    B = BT.Batch(geoms, params)
    if tuned:
        t = B.tune()
        assert len(t["candidates"]) >= 3
        assert 0 <= t["shape"] < 3 and t["grid"] >= 1 and t["ms_per_step"] > 0
    st = B.run()
    assert not st.any()
    info = B.info
    assert info["n"] == 3 and info["run_ms"] > 0 and info["kernel_launches"] >= RUN["steps"]
    for v, g, p in zip(B.variants, geoms, params):
        ref, ref_acc = individual(g, p)
        got = v.evaluate()
        assert np.array_equal(v.get_acc(), ref_acc)
        for k in ("gamma", "gammaCore", "zeta", "maxToMean", "lowCore"):
            assert got["metrics"][k] == ref["metrics"][k], k
        assert got["hist"] == ref["hist"]


def test_shapes_and_grids_agree():
    geoms, params = variants()
    params = [dict(p, storage="f16") for p in params]
    B = BT.Batch(geoms, params)
    out = []
    for shape, grid, group in ((0, 10 ** 6, 0), (1, 7, 0), (2, 3, 0), (0, 300, 1.0), (1, 5, 2e6)):
        B.reset()
        B.set_grouping(group)           # 1 byte: every variant its own group
        B.set_shape(shape, grid)
        B.run()
        assert B.info["n_groups"] == (3 if group == 1.0 else B.info["n_groups"])
        out.append([v.get_acc() for v in B.variants])
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)


def test_unstable_variant_stops_alone():
    geoms, params = variants()
    params[1] = dict(params[1], u=0.0)          # zero inflow: sigma = 0/0, the run goes non-finite
    B = BT.Batch(geoms, params)
    st = B.run()
    assert st[1] == RUN["every"] and st[0] == 0 and st[2] == 0
    for i in (0, 2):
        ref, ref_acc = individual(geoms[i], params[i])
        assert np.array_equal(B.variants[i].get_acc(), ref_acc)


def test_batch_argument_errors():
    geoms, params = variants()
    with pytest.raises(E.AirboxError):
        BT.Batch(geoms, [params[0], dict(params[1], steps=60), params[2]])
    with pytest.raises(E.AirboxError):
        BT.Batch(geoms, [dict(p, storage="f64") for p in params])


def test_batches_larger_than_one_launch():
    """More variants than one launch carries (96): the steps are split over several launches."""
    spec = ag.AirboxSpec(**SMALL)
    g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params()})
    run = dict(RUN, steps=60, avg=20, every=30, storage="f16")
    params = [dict(run, K=1.0 + 0.05 * i) for i in range(100)]
    B = BT.Batch([g] * 100, params)
    B.tune()
    assert not B.run().any()
    for i in (0, 95, 96, 99):
        _, ref_acc = individual(g, params[i])
        assert np.array_equal(B.variants[i].get_acc(), ref_acc), i
