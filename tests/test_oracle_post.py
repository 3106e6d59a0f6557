"""CPU checks of the oracle's post-processing restatement (field3d, cut
planes, streamlines; src/engine.js:662-680, 698-758) and of the warm-start
resampling restatement, before they serve as checkers of the GPU kernels."""
import math

import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from oracle import oracle as O
from oracle import warmstart_ref as R_

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})
RUN = dict(K=3, aniso=10, u=0.06, tau=0.51)


@pytest.fixture(scope="module")
def solved():
    spec = ag.AirboxSpec(**SMALL)
    og = O.prepare(ag.build_airbox(spec), spec.prepare_params())
    S = O.OracleSim(og, RUN)
    acc, _ = S.simulate(200, 100, 50)
    return og, S, acc


def test_js_hypot_and_round():
    L = O.lib()
    rng = np.random.default_rng(0)
    for x, y, z in rng.standard_normal((200, 3)) * 10 ** rng.uniform(-5, 5, (200, 1)):
        h = L.ora_js_hypot3(x, y, z)
        assert abs(h - math.hypot(x, y, z)) <= 4.5e-16 * h   # within 2 ulp of a correctly rounded hypot
    assert L.ora_js_hypot3(0.0, 0.0, 0.0) == 0.0
    assert L.ora_js_hypot3(3.0, 4.0, 12.0) == 13.0
    assert math.isinf(L.ora_js_hypot3(float("inf"), 1.0, float("nan")))  # V8: Infinity wins over NaN
    L.ora_js_round.restype = __import__("ctypes").c_double
    L.ora_js_round.argtypes = [__import__("ctypes").c_double]
    assert [L.ora_js_round(v) for v in (2.5, -2.5, 0.49999999999999994, -0.5, 1.5)] == [3.0, -2.0, 0.0, -0.0, 2.0]


def test_field3d_structure(solved):
    og, S, acc = solved
    (spd, pst, loss), kB, pin, rr = S.field3d(acc)
    nx, ny, nz = spd.shape
    fl = np.zeros(og.nx * og.ny * og.nz, bool)
    cid = np.full(fl.size, -1)
    cid[S.cells()] = np.arange(S.NF)
    fl[S.cells()] = True
    fl = fl.reshape(nx, ny, nz)
    assert np.isnan(spd[:, :, :kB]).all()
    assert np.isnan(spd[~fl]).all() and np.isfinite(spd[fl][..., None][:, :]).any()
    a = acc.reshape(4, -1)
    c = cid.reshape(nx, ny, nz)
    ii, jj, kk = np.nonzero(fl & (np.arange(nz)[None, None, :] >= kB))
    idx = c[ii, jj, kk]
    ref = np.hypot(np.hypot(a[0, idx].astype(np.float64), a[1, idx]), a[2, idx]) / RUN["u"]
    assert np.allclose(spd[ii, jj, kk], ref, rtol=1e-6, atol=0)
    # static pressure is measured from the mean density of layer jb (the evaluate() reference of zeta)
    dc = np.ctypeslib.as_array(og.g.dc, shape=(ny,)).astype(np.float64)
    jb = int(np.argmax(dc >= og.g.pleat + 2 * og.g.h))
    cells = c[:, jb, :][fl[:, jb, :]]
    assert abs(rr - a[3, cells].astype(np.float64).mean()) < 1e-12
    assert np.isfinite(pin) and abs(rr - 1) < 0.05


def test_planes_and_streamlines(solved):
    og, S, acc = solved
    pl, (ic, jc, jlow) = S.planes(acc)
    nx, ny, nz = og.nx, og.ny, og.nz
    P, Q = nx * nz, nz * ny
    assert pl.size == 6 * P + 3 * Q
    sp_in = pl[:P]
    assert np.isfinite(sp_in).sum() > 10 and np.nanmax(sp_in) > 0.5
    assert 0 <= ic < nx and 0 <= jc < ny and 0 <= jlow < ny
    pts, spd, off = S.streamlines(acc)
    assert off[0] == 0 and np.all(np.diff(off) >= 2) and off[-1] == spd.size == pts.size // 3
    assert len(off) - 1 <= 221 and np.all(np.isfinite(pts))
    # every line starts in front of the box, at the inlet
    starts = pts.reshape(-1, 3)[off[:-1]]
    assert np.ptp(starts[:, 2]) < 1e-3 or np.ptp(starts[:, 1]) < 1e-3 or np.ptp(starts[:, 0]) < 1e-3


@pytest.mark.parametrize("n,R", [(160, 64), (45, 64), (64, 64), (97, 16), (10, 16)])
def test_warmstart_footprints_cover_the_grid(n, R):
    fp = [R_.footprint(a, n, R) for a in range(R)]
    assert all(0 <= a < b <= n for a, b in fp)
    if n >= R:   # a partition of [0, n)
        assert fp[0][0] == 0 and fp[-1][1] == n and all(fp[i][1] == fp[i + 1][0] for i in range(R - 1))
    else:        # every voxel takes one cell, in order
        assert all(b - a == 1 for a, b in fp) and [a for a, _ in fp] == sorted(a for a, _ in fp)


def test_warmstart_features_of_a_synthetic_grid():
    cls = np.zeros((20, 12, 18), np.uint8)
    cls[2:18, 2:10, 1:17] = 1
    cls[5:9, 4:7, 1] = 2
    cls[2:18, 2, 1:17] = 3
    cls[2:18, 3:5, 1:17] = 4
    x, d = R_.features(cls, 8, 3.0)
    assert x.shape == (9, 8, 8, 8) and x.dtype == np.float32
    assert np.all((0 <= x[:4]) & (x[:4] <= 1))
    assert np.allclose(x[5], 1.0) and np.allclose(x[6], 20 / 128)
    # fractions are exact footprint counts: total fluid cells is recovered
    n = R_._counts(20, 12, 18, 8)
    assert int(round(float((x[0].astype(np.float64) * n).sum()))) == int((cls > 0).sum())
    assert (d[x[0] < 0.5] == 0).all() and (d[x[0] >= 0.5] > 0).all()


def test_warmstart_coordinate_channels():
    cls = np.zeros((20, 12, 18), np.uint8)
    cls[2:18, 2:10, 1:17] = 1
    x, _ = R_.features(cls, 8, 3.0, coords=True)
    assert x.shape == (12, 8, 8, 8)
    c = (np.arange(8) + 0.5) / 8
    assert np.allclose(x[9], c[:, None, None]) and np.allclose(x[10], c[None, :, None])
    assert np.allclose(x[11], c[None, None, :])
    assert [l[0] for l in R_.conv_layers(16, 4, 12)][0] == 12
