"""GPU parity: libairbox.so (through the C ABI) against the oracle, the C
restatement of src/engine.js, on the same seeded geometries.

* voxel masks, opening, flood and outlet: bit-exact;
* ``f32exact`` storage (float32 populations, cpuStep's float64 arithmetic):
  populations bit-identical to cpuStep after every tested step count, and the
  same progress history and KPIs;
* ``f64``: bit-identical to the float64 oracle;
* ``f32`` (the WGSL lbm_step contract): the reference's own self-test bound
  (max |df| < 1e-3 after 12 steps, src/engine.js:597-611,772) and a tighter one,
  time-averaged fields within 1e-3 relative L2 and KPIs within 0.5 %.
"""
import os

import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu

RUN = dict(K=3.0, aniso=10.0, u=0.06, tau=0.51)
NT = os.cpu_count() or 1

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})


def geom_cases():
    cases = {
        "small_baffle": (ag.AirboxSpec(**SMALL), {}),
        "config1": (ag.config1_spec(), {}),
        "yaw_seed3": (ag.random_spec(3, dx=4.0), {}),
        "yaw_seed11": (ag.random_spec(11, dx=3.5), {}),
        "fine_cells": (ag.AirboxSpec(Lx=96.17, Ly=71.43, Lz=80.29, t=2.93, d_in=30.11, stub=15.37, pleat=30.0,
                                     dx=2.5, baffle={"z": 33.71, "x0": 40.13, "x1": 93.24, "y0": 55.07}), {}),
    }
    spec = ag.config1_spec()
    cases["outlet_plenum"] = (spec, {"outlet": {"enabled": True, "center": [120.0, 0.0, 90.0], "diameter": 60.0,
                                                "height": 20.0}})
    cases["click"] = (spec, {"click": [120.0, 77.0, -30.0]})
    # three holes in the front slice: the stub's and two tubes'; the click picks a tube, or the largest wins
    cases["tubes_largest"] = (spec, {"_tubes": True})
    cases["tubes_click_small"] = (spec, {"_tubes": True, "click": [210.0, 70.0, -30.0]})
    cases["tubes_click_left"] = (spec, {"_tubes": True, "click": [25.0, 64.0, -30.0]})
    # no distance compares below Infinity: the first component in scan order stays chosen, not the largest
    cases["tubes_click_nan"] = (spec, {"_tubes": True, "click": [float("nan"), 70.0, -30.0]})
    return cases


CASES = geom_cases()


def airbox_with_tubes(spec):
    """The airbox plus two square tubes, capped at the back, standing in front of its inlet wall beside the
    stub (disjoint closed solids): the fine slice behind the front-most point then holds three holes, and a
    click on a tube makes prepare choose that tube's (smaller) hole as the opening."""
    z0 = -spec.stub
    z1 = z0 + 10.0
    parts = [ag.build_airbox(spec)]
    for x0, y0, w, wall in ((10.0, 50.0, 40.0, 8.0), (195.0, 55.0, 30.0, 8.0)):
        x1, y1 = x0 + w, y0 + w
        walls = [(x0, x0 + wall, y0, y1), (x1 - wall, x1, y0, y1), (x0 + wall, x1 - wall, y0, y0 + wall),
                 (x0 + wall, x1 - wall, y1 - wall, y1)]
        parts += [ag._box(a, b, c, d, z0, z1 - 3.0).reshape(-1, 9) for a, b, c, d in walls]
        parts.append(ag._box(x0, x1, y0, y1, z1 - 3.0, z1).reshape(-1, 9))
    return np.concatenate(parts).astype(np.float32)


def prep_both(spec, extra=None, **kw):
    extra = dict(extra or {})
    tris = airbox_with_tubes(spec) if extra.pop("_tubes", False) else ag.build_airbox(spec)
    p = {**spec.prepare_params(), **extra}
    og = O.prepare(tris, p, keep_fine=kw.get("keep_fine", False), max_cells=kw.get("max_cells", 4.5e6))
    g = E.prepare({"tris": tris, **p, "maxCells": kw.get("max_cells", 4.5e6)})
    return og, g


@pytest.mark.parametrize("name", list(CASES))
def test_geometry_bit_exact(name):
    spec, extra = CASES[name]
    og, g = prep_both(spec, extra, keep_fine=True)
    assert (g.nx, g.ny, g.nz) == (og.nx, og.ny, og.nz)
    assert np.array_equal(g.fine(), og.fine()), "fine voxel grid"
    assert np.array_equal(g.solid, og.solid()), "solid"
    assert np.array_equal(g.fluid, og.fluid()), "fluid"
    assert np.array_equal(g.opening, og.opening()), "opening"
    assert np.array_equal(g.outlet, og.outlet()), "outlet"
    assert np.array_equal(g.dc, og.dc()) and np.array_equal(g.xc, og.xc()) and np.array_equal(g.zc, og.zc())
    i = g.info
    for a, b in [("nf", "nf"), ("top", "top"), ("jm", "jm"), ("af", "Af"), ("n_open", "nOpen"),
                 ("n_holes", "nHoles"), ("kw0", "kw0"), ("kf", "kf"), ("n_out", "nOut")]:
        assert getattr(i, a) == getattr(og.g, b), a
    assert list(i.origin) == list(og.g.origin) and list(i.mn) == list(og.g.mn) and list(i.mx) == list(og.g.mx)


def bulk_ns(S_or, NF):
    """The self-test's partial bounce-back field: every 17th bulk cell set to 1
    (src/engine.js:600), plus some fractional values."""
    ns = np.zeros(NF, np.float32)
    flag = S_or.flag()
    for a in range(0, NF, 17):
        if flag[a] == 0:
            ns[a] = 1.0
    for a in range(5, NF, 53):
        if flag[a] == 0:
            ns[a] = 0.37
    return ns


def oracle_steps(S, f, n, kind, ns=None, acc=None):
    for _ in range(n):
        f = S.step(f, acc=acc, ns=ns, kind=kind, nthreads=NT)
    return f


@pytest.mark.parametrize("with_ns", [False, True])
def test_f32exact_steps_bit_identical(with_ns):
    og, g = prep_both(ag.AirboxSpec(**SMALL))
    So = O.OracleSim(og, RUN)
    ns = bulk_ns(So, So.NF) if with_ns else None
    Sg = E.Simulation(g, {**RUN, "storage": "f32exact"}, ns=ns)
    assert Sg.NF == So.NF and Sg.Ain == So.S.Ain and Sg.Af == So.S.Af and Sg.sig == So.S.sig
    f = So.f0()
    done = 0
    for n in (1, 1, 1, 9, 28):
        f = oracle_steps(So, f, n, "f32", ns)
        Sg.step(n)
        done += n
        got = Sg.get_f()
        assert np.array_equal(got, f), f"populations differ after {done} steps (max {np.abs(got - f).max()})"


def test_f32exact_accumulation_bit_identical():
    og, g = prep_both(ag.AirboxSpec(**SMALL))
    So = O.OracleSim(og, RUN)
    Sg = E.Simulation(g, {**RUN, "storage": "f32exact"})
    f = So.f0()
    acc = np.zeros(4 * So.NF, np.float32)
    f = oracle_steps(So, f, 7, "f32")
    f = oracle_steps(So, f, 13, "f32", acc=acc)
    Sg.step(7)
    Sg.step(13, accumulate=True)
    want = (acc.astype(np.float64) / 13).astype(np.float32)
    assert np.array_equal(Sg.get_acc(), want)
    assert np.array_equal(Sg.get_f(), f)


def test_f64_steps_bit_identical():
    og, g = prep_both(ag.AirboxSpec(**SMALL))
    So = O.OracleSim(og, RUN)
    Sg = E.Simulation(g, {**RUN, "storage": "f64"})
    f = So.f0(np.float64)
    f = oracle_steps(So, f, 25, "f64")
    Sg.step(25)
    assert np.array_equal(Sg.get_f(), f.astype(np.float32))


@pytest.mark.parametrize("storage,tol", [("f32", 1e-5), ("f16", 2e-3), ("bf16", 2e-2)])
def test_reference_self_test(storage, tol):
    """gpuSelfTest (src/engine.js:597-611): two variants (plain, and ns = 1 on
    every 17th bulk cell), 12 steps from w_i, max |df| over every 7th entry."""
    og, g = prep_both(ag.config1_spec())
    So = O.OracleSim(og, RUN)
    md = 0.0
    for ns in (None, bulk_ns(So, So.NF)):
        f = oracle_steps(So, So.f0(), 12, "f32", ns)
        Sg = E.Simulation(g, {**RUN, "storage": storage, "allowBf16": True}, ns=ns)
        Sg.step(12)
        d = np.abs(Sg.get_f() - f)[::7]
        md = max(md, float(d.max()))
    assert md < 1e-3, md          # the reference's acceptance bound (src/engine.js:772)
    assert md < tol, md


def run_both(spec, storage, steps, avg, every, extra_run=None):
    og, g = prep_both(spec)
    run = {**RUN, **(extra_run or {}), "steps": steps, "avg": avg, "every": every}
    So = O.OracleSim(og, run)
    acc_o, hist_o = So.simulate(steps, avg, every, nthreads=NT)
    m_o, fmap_o = So.evaluate(acc_o)
    Sg = E.Simulation(g, {**run, "storage": storage, "allowBf16": True})
    Sg.run()
    res = Sg.evaluate()
    return So, Sg, acc_o, hist_o, m_o, fmap_o, res


def test_f32exact_full_run_matches_oracle():
    So, Sg, acc_o, hist_o, m_o, fmap_o, res = run_both(ag.AirboxSpec(**SMALL), "f32exact", 600, 200, 150)
    assert np.array_equal(Sg.get_acc(), acc_o)
    assert np.allclose(np.array(res["hist"]), hist_o, rtol=1e-12, atol=1e-15)
    for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean", "zeta"):
        assert res["metrics"][k] == pytest.approx(m_o[k], rel=1e-12, abs=1e-15), k
    fm = res["fmap"].reshape(fmap_o.shape)
    assert np.array_equal(np.isnan(fm), np.isnan(fmap_o))
    assert np.allclose(fm[~np.isnan(fm)], fmap_o[~np.isnan(fmap_o)], rtol=1e-6)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_f32_full_run_within_tolerance():
    """FP32 GPU vs the cpuStep oracle on a 600-step run: time-averaged u and rho
    within 1e-3 relative L2, KPIs within 0.5 %."""
    So, Sg, acc_o, hist_o, m_o, fmap_o, res = run_both(ag.AirboxSpec(**SMALL), "f32", 600, 200, 150)
    acc = Sg.get_acc().reshape(4, -1)
    ao = acc_o.reshape(4, -1)
    for c in range(3):
        assert rel_l2(acc[c], ao[c]) < 1e-3, c
    assert rel_l2(acc[3] - 1, ao[3] - 1) < 1e-3
    for k in ("gamma", "gammaCore", "zeta", "maxToMean"):
        assert res["metrics"][k] == pytest.approx(m_o[k], rel=5e-3), k


@pytest.mark.parametrize("name", ["no_opening", "same_axis", "grid_too_large", "bad_outlet", "lid_too_low",
                                  "opening_too_small"])
def test_prepare_errors_match_reference(name):
    spec = ag.config1_spec()
    tris = ag.build_airbox(spec)
    p = spec.prepare_params()
    kw = {}
    if name == "opening_too_small":                  # a click on the small tube's hole at 5 mm cells
        tris = airbox_with_tubes(spec)
        p.update(click=[210.0, 70.0, -30.0], dx=5.0)
    elif name == "no_opening":
        p["inletAxis"], p["inletSign"] = 0, -1        # a side face without a hole
    elif name == "same_axis":
        p["inletAxis"] = 1
    elif name == "grid_too_large":
        kw["max_cells"] = 1000.0
    elif name == "bad_outlet":
        p["outlet"] = {"enabled": True, "center": [5000.0, 0.0, 5000.0], "diameter": 10.0, "height": 20.0}
    elif name == "lid_too_low":
        p["outlet"] = {"enabled": True, "center": [120.0, 0.0, 90.0], "diameter": 60.0, "height": 0.5}
    with pytest.raises(O.OracleError) as eo:
        O.prepare(tris, p, max_cells=kw.get("max_cells", 4.5e6))
    with pytest.raises(E.AirboxError) as eg:
        E.prepare({"tris": tris, **p, "maxCells": kw.get("max_cells", 4.5e6)})
    assert eg.value.code == eo.value.code
    assert str(eg.value) == str(eo.value)


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_tma_pipeline_matches_direct_kernel(storage, monkeypatch):
    """The TMA-fed step kernel and the direct-load kernel run the same
    collision on the same data: their states agree after odd and even steps,
    with and without averaging, to float32 rounding (one unit of the stored
    deviation for the 16-bit formats: the two kernels may contract a
    multiply-add differently before the value is rounded to 16 bits)."""
    tol = {"f32": 1e-6, "f16": 1.3e-4, "bf16": 1e-3}[storage]
    og, g = prep_both(ag.config1_spec())
    So = O.OracleSim(og, RUN)
    ns = bulk_ns(So, So.NF)
    out = {}
    for tma in (True, False):
        if tma:
            monkeypatch.setenv("ABX_TMA", "1")
        else:
            monkeypatch.delenv("ABX_TMA", raising=False)
        for with_ns in (False, True):
            S = E.Simulation(g, {**RUN, "storage": storage, "allowBf16": True}, ns=ns if with_ns else None)
            assert S.info.tma_pipeline == (1 if tma else 0)
            S.step(7)
            S.step(6, accumulate=True)
            out[(tma, with_ns)] = (S.get_f(), S.get_acc())
    for with_ns in (False, True):
        fa, aa = out[(True, with_ns)]
        fb, ab = out[(False, with_ns)]
        assert np.abs(fa - fb).max() < tol
        assert np.abs(aa - ab).max() < 1e-5


@pytest.mark.parametrize("storage", ["f32exact", "f32", "f16", "bf16"])
def test_zero_inflow_fails_like_the_reference(storage):
    """u = 0 makes the filter coefficient 0/0 (src/engine.js:258): Math.min keeps the NaN, the fields go
    non-finite and the first progress check reports the instability, as in the oracle."""
    og, g = prep_both(ag.AirboxSpec(**SMALL))
    run = dict(K=3.0, aniso=10.0, u=0.0, tau=0.51, steps=200, avg=50, every=50)
    with pytest.raises(O.OracleError) as eo:
        O.OracleSim(og, run).simulate(200, 50, 50, nthreads=NT)
    with pytest.raises(E.AirboxError) as eg:
        E.Simulation(g, {**run, "storage": storage, "allowBf16": True}).run()
    assert eg.value.code == 10 and str(eg.value) == str(eo.value)


@pytest.mark.parametrize("storage", ["f32exact", "f32", "f16"])
def test_instability_reported_like_the_reference(storage):
    """progressInfo's check (src/engine.js:334-335): a run that blows up fails
    with the reference's message; with cpuStep's exact arithmetic at the same
    step as the oracle."""
    og, g = prep_both(ag.AirboxSpec(**SMALL))
    run = dict(K=3.0, aniso=10.0, u=0.45, tau=0.5001, steps=3000, avg=100, every=50)
    So = O.OracleSim(og, run)
    with pytest.raises(O.OracleError) as eo:
        So.simulate(3000, 100, 50, nthreads=NT)
    S = E.Simulation(g, {**run, "storage": storage, "allowBf16": True})
    with pytest.raises(E.AirboxError) as eg:
        S.run()
    assert eg.value.code == 10 and "Rechnung instabil bei Schritt" in str(eg.value)
    if storage == "f32exact":
        assert str(eg.value) == str(eo.value)
    # the same handle runs again after a reset
    S.reset()
    S.step(5)
