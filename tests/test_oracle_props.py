"""Known-answer properties of the oracle's LBM (src/engine.js:266-321), on CPU.

The reference ships no golden vectors for the step, so these pin what the
physics fixes: a fluid at rest with no inflow stays at the equilibrium w_i,
a geometry mirror-symmetric in x gives mirror-symmetric averages, and the
float64 and float32-storage oracles agree to float32 rounding."""
import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from oracle import oracle as O

SYM = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0)


def geom(spec):
    return O.prepare(ag.build_airbox(ag.AirboxSpec(**spec)), ag.AirboxSpec(**spec).prepare_params())


def test_rest_state_is_stationary():
    """A vanishing inflow (1e-9) leaves every population at w_i to float32
    resolution.  (u = 0 itself makes the reference's Darcy coefficient
    K u0^2 / (2 uface Lp) a 0/0, src/engine.js:259; see the next test.)"""
    og = geom(SYM)
    S = O.OracleSim(og, dict(K=3, aniso=10, u=1e-9, tau=0.51))
    f0 = S.f0()
    f = f0
    for _ in range(20):
        f = S.step(f, nthreads=2)
    assert np.abs(f - f0).max() < 2e-7


def test_zero_inflow_is_reported_unstable():
    og = geom(SYM)
    S = O.OracleSim(og, dict(K=3, aniso=10, u=0.0, tau=0.51))
    with pytest.raises(O.OracleError) as e:
        S.simulate(100, 50, 50, nthreads=2)
    assert "Rechnung instabil bei Schritt 50" in str(e.value)


def test_mirror_symmetry_of_the_averages():
    spec = dict(SYM, Lx=130.0, t=3.11)   # hole centred in x, no baffle
    tris = ag.build_airbox(ag.AirboxSpec(**spec))
    p = ag.AirboxSpec(**spec).prepare_params()
    og = O.prepare(tris, p)
    fl = og.fluid().reshape(og.nx, og.ny, og.nz)
    if not np.array_equal(fl, fl[::-1]):
        pytest.skip("voxelization not mirror-symmetric at this size")
    S = O.OracleSim(og, dict(K=3, aniso=10, u=0.06, tau=0.51))
    acc, _ = S.simulate(120, 60, 60, nthreads=2)
    cells = S.cells()
    NF = S.NF
    full = np.full((4, og.nx * og.ny * og.nz), np.nan)
    full[:, cells] = acc.reshape(4, NF)
    full = full.reshape(4, og.nx, og.ny, og.nz)
    m = ~np.isnan(full[0])
    ux, uy, uz, rho = full
    assert np.allclose(ux[m], -ux[::-1][m], atol=1e-6)
    for a in (uy, uz, rho):
        assert np.allclose(a[m], a[::-1][m], atol=1e-6)


def test_float64_and_float32_oracles_agree():
    og = geom(SYM)
    S = O.OracleSim(og, dict(K=3, aniso=10, u=0.06, tau=0.51))
    f32, f64 = S.f0(), S.f0(np.float64)
    for _ in range(30):
        f32 = S.step(f32, kind="f32", nthreads=2)
        f64 = S.step(f64, kind="f64", nthreads=2)
    assert np.abs(f32 - f64).max() < 1e-6


def test_reference_self_test_structure_on_the_oracle():
    """gpuSelfTest's second variant (ns = 1 on every 17th bulk cell) changes the
    flow, and its float32-local form (WGSL semantics) stays within the
    reference's 1e-3 acceptance bound of the float64-local form."""
    og = geom(SYM)
    S = O.OracleSim(og, dict(K=3, aniso=10, u=0.06, tau=0.51))
    ns = np.zeros(S.NF, np.float32)
    flag = S.flag()
    for a in range(0, S.NF, 17):
        if flag[a] == 0:
            ns[a] = 1.0
    fa, fb, fl = S.f0(), S.f0(), S.f0()
    for _ in range(12):
        fa = S.step(fa, nthreads=2)
        fb = S.step(fb, ns=ns, nthreads=2)
        fl = S.step(fl, ns=ns, kind="f32l", nthreads=2)
    assert np.abs(fa - fb).max() > 1e-4
    assert np.abs(fl - fb)[::7].max() < 1e-3


def test_instability_is_reported_with_the_reference_message():
    og = geom(SYM)
    S = O.OracleSim(og, dict(K=3, aniso=10, u=0.45, tau=0.5001))
    with pytest.raises(O.OracleError) as e:
        S.simulate(3000, 100, 50, nthreads=2)
    assert "Rechnung instabil bei Schritt" in str(e.value)
