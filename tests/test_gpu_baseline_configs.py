"""GPU parity on the benchmark configurations themselves, not only on small
cases: libairbox.so (through the C ABI) against the oracle (the C restatement
of src/engine.js) and against the GPU's own float64 run.

* config1 (240x120x180 mm airbox, dx 4 mm) on the reference's full schedule
  (6000 steps, last 2000 averaged, progress every 150; src/engine.js:341-358):
  ``f32exact`` averages bit-identical to the oracle's simulate(), history and
  KPIs to 1e-12; ``f32`` time-averaged u and rho - 1 within 1e-3 relative L2
  of the oracle and KPIs within 0.5 % (the float32 contract of the WGSL
  lbm_step, src/engine.js:378-450).
* config2 (seeded airbox 1000, dx 1.5 mm, 1.65 M fluid cells) and config3
  (512x256x384 cells, 39.2 M fluid cells) geometry: every mask, the opening
  and the scalars bit-exact against the oracle's prepare() with the 4.5 M cell
  cap lifted; the fluid-cell order of the device layout checked through
  cpuStep-exact steps (bit-identical populations).
* config2 on its full schedule in every storage: the float64 run is
  bit-identical to the float64 oracle step by step, and the float32, float16
  and bfloat16 runs keep every KPI within 0.5 % of it.
* config3: the decorrelation horizon.  float32 and float16 runs from w_i stay
  within 1e-3 relative L2 of the float64 run (fields averaged over 100 steps)
  up to step 2000; beyond it the unsteady flow's trajectories drift apart.
"""
import os

import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
RUN1 = dict(K=3.0, aniso=10.0, u=0.06, tau=0.51, steps=6000, avg=2000, every=150)
RUN3 = dict(K=3.0, aniso=10.0, u=0.05, tau=0.505, steps=20000, avg=5000, every=500)
KPIS = ("gamma", "gammaCore", "maxToMean", "zeta")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def host_memory_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 2 ** 20
    except OSError:
        pass
    return 0.0


# ------------------------------------------------------------------ config1, full schedule
@pytest.fixture(scope="module")
def config1_oracle():
    spec = ag.config1_spec()
    tris = ag.build_airbox(spec)
    p = spec.prepare_params()
    og = O.prepare(tris, p)
    So = O.OracleSim(og, RUN1)
    acc, hist = So.simulate(RUN1["steps"], RUN1["avg"], RUN1["every"], nthreads=NT)
    m, fmap = So.evaluate(acc)
    g = E.prepare({"tris": tris, **p})
    return g, So, acc, hist, m, fmap


def test_config1_full_schedule_f32exact_bit_identical(config1_oracle):
    g, So, acc_o, hist_o, m_o, fmap_o = config1_oracle
    S = E.Simulation(g, {**RUN1, "storage": "f32exact"})
    assert S.NF == So.NF
    S.run()
    res = S.evaluate()
    assert np.array_equal(S.get_acc(), acc_o), "time averages differ from the oracle's simulate()"
    assert len(res["hist"]) == len(hist_o)
    assert np.allclose(np.array(res["hist"]), hist_o, rtol=1e-12, atol=1e-15)
    for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean", "zeta"):
        assert res["metrics"][k] == pytest.approx(m_o[k], rel=1e-12, abs=1e-15), k


def test_config1_full_schedule_f32_within_tolerance(config1_oracle):
    """float32 collision (the WGSL lbm_step arithmetic): time-averaged u and
    rho - 1 within 1e-3 relative L2 of the oracle, KPIs within 0.5 %."""
    g, So, acc_o, hist_o, m_o, fmap_o = config1_oracle
    S = E.Simulation(g, {**RUN1, "storage": "f32"})
    S.run()
    res = S.evaluate()
    a = S.get_acc().reshape(4, -1).astype(np.float64)
    b = acc_o.reshape(4, -1).astype(np.float64)
    assert rel_l2(a[:3], b[:3]) < 1e-3
    assert rel_l2(a[3] - 1, b[3] - 1) < 1e-3
    for k in KPIS:
        assert res["metrics"][k] == pytest.approx(m_o[k], rel=5e-3), k


# ------------------------------------------------------------------ config2 / config3 geometry
def large_cases():
    return {"config2": ag.random_spec(1000, dx=1.5), "config3": ag.grid_spec(512, 256, 384, dx=0.6)}


@pytest.mark.parametrize("name", ["config2", "config3"])
def test_large_geometry_bit_exact(name):
    """prepare() at the benchmark sizes (cell cap lifted, as the reference's
    4.5 M cap at src/engine.js:124 allows neither): fine voxel grid (config2),
    solid / fluid / opening / outlet masks and every scalar equal to the
    oracle's."""
    if name == "config3" and host_memory_gb() < 24:
        pytest.skip("the config3 oracle needs about 16 GB of host memory")
    spec = large_cases()[name]
    tris = ag.build_airbox(spec)
    p = spec.prepare_params()
    og = O.prepare(tris, p, max_cells=1e10, keep_fine=(name == "config2"))
    g = E.prepare({"tris": tris, **p, "maxCells": 1e10})
    assert (g.nx, g.ny, g.nz) == (og.nx, og.ny, og.nz)
    if name == "config2":
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
    # the device layout (kpad, segments, 32-bit element offsets, compact cell order) through two cpuStep-exact
    # steps: populations in the reference's fluid-cell order, bit-identical
    So = O.OracleSim(og, RUN3)
    Sg = E.Simulation(g, {**RUN3, "storage": "f32exact"})
    assert Sg.NF == So.NF and Sg.Ain == So.S.Ain and Sg.Af == So.S.Af and Sg.sig == So.S.sig
    f = So.f0()
    for _ in range(2):
        f = So.step(f, kind="f32", nthreads=NT)
    Sg.step(2)
    got = Sg.get_f()
    assert np.array_equal(got, f), f"populations differ after 2 steps (max {np.abs(got - f).max()})"


# ------------------------------------------------------------------ config2, every storage
@pytest.fixture(scope="module")
def config2():
    spec = ag.random_spec(1000, dx=1.5)
    tris = ag.build_airbox(spec)
    p = spec.prepare_params()
    return spec, tris, p, E.prepare({"tris": tris, **p, "maxCells": 1e10})


def test_config2_f64_bit_identical_to_fp64_oracle(config2):
    spec, tris, p, g = config2
    og = O.prepare(tris, p, max_cells=1e10)
    So = O.OracleSim(og, RUN1)
    Sg = E.Simulation(g, {**RUN1, "storage": "f64"})
    f = So.f0(np.float64)
    for _ in range(12):
        f = So.step(f, kind="f64", nthreads=NT)
    Sg.step(12)
    assert np.array_equal(Sg.get_f(), f.astype(np.float32))


@pytest.fixture(scope="module")
def config2_runs(config2):
    spec, tris, p, g = config2
    out = {}
    for st in ("f64", "f32", "f16", "bf16"):
        S = E.Simulation(g, {**RUN1, "storage": st, "allowBf16": True})
        S.run()
        out[st] = (S.evaluate()["metrics"], S.get_acc().reshape(4, -1).astype(np.float64))
        del S
    return out


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_config2_kpis_within_half_percent_of_f64(config2_runs, storage):
    """config2 on its full 6000/2000 schedule: every KPI of the float32, float16
    and bfloat16 runs within 0.5 % of the float64 run; float32 and float16
    time-averaged fields within 1e-3 relative L2 of it."""
    m64, a64 = config2_runs["f64"]
    m, a = config2_runs[storage]
    for k in KPIS:
        assert m[k] == pytest.approx(m64[k], rel=5e-3), (k, m[k], m64[k])
    if storage != "bf16":
        assert rel_l2(a[:3], a64[:3]) < 1e-3
        assert rel_l2(a[3] - 1, a64[3] - 1) < 1e-3


def test_bf16_requires_opt_in(config2):
    spec, tris, p, g = config2
    with pytest.raises(E.AirboxError) as ei:
        E.Simulation(g, {**RUN1, "storage": "bf16"})
    assert ei.value.code == 20 and "bfloat16" in str(ei.value) and "ABX_RUN_ALLOW_BF16" in str(ei.value)


# ------------------------------------------------------------------ config3, decorrelation horizon
HORIZON = 2000


def test_config3_decorrelation_horizon():
    """config3 (tau 0.505, u 0.05) from w_i: the float32 and float16 runs' fields,
    averaged over steps HORIZON..HORIZON+100, are within 1e-3 relative L2 of
    the float64 run's (u and rho - 1).  Over the full 20000-step schedule
    the unsteady trajectories drift apart (the fields then differ by more,
    while the time-averaged KPIs stay within 0.5 %: the precision study)."""
    spec = ag.grid_spec(512, 256, 384, dx=0.6)
    g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
    acc = {}
    for st in ("f64", "f32", "f16"):
        S = E.Simulation(g, {**RUN3, "storage": st})
        S.step(HORIZON)
        S.step(100, True)
        acc[st] = S.get_acc().reshape(4, -1).astype(np.float64)
        del S
    for st in ("f32", "f16"):
        assert rel_l2(acc[st][:3], acc["f64"][:3]) < 1e-3, st
        assert rel_l2(acc[st][3] - 1, acc["f64"][3] - 1) < 1e-3, st
