"""abx_voxelize_static: the parity voxelizer for callers that cannot allocate
GPU memory (their memory pool owns every device byte), checked through the C
ABI against the voxel grid of the allocating path (abx_prepare, read back
with abx_geom_get_fine).

The caller's device buffers come from PyTorch here.  The entry point shares
one fixed scratch array across calls, so the test runs several calls in a row
on different meshes and grid sizes: no call may see the previous call's
leftovers.  It passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from airboxcalc_gb300 import _abi as A
from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E

pytestmark = pytest.mark.gpu

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})


def local_triangles(g: E.Geometry, tris: np.ndarray) -> np.ndarray:
    """The frame transform prepare() applies (float64 arithmetic, float32 result)."""
    fr = g.fr
    P = np.asarray(tris, np.float32).reshape(-1, 3).astype(np.float64)
    a, b = P[:, fr.oAx], -fr.si * P[:, fr.iAx]
    X = fr.cy * a + fr.sy * b
    D = -fr.sd * (P[:, fr.dAx] - fr.seal)
    Z = -fr.sy * a + fr.cy * b
    return np.stack([X, D, Z], 1).astype(np.float32).ravel()


def static_voxelize(torch, local: np.ndarray, origin, h, nx, ny, nz) -> np.ndarray:
    d_tris = torch.from_numpy(local).cuda()
    d_vox = torch.full((nx * ny * nz,), 7, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    rc = A.load().abx_voxelize_static(C.c_void_p(d_tris.data_ptr()), local.size, (C.c_double * 3)(*origin), h,
                                      nx, ny, nz, C.c_void_p(d_vox.data_ptr()), None)
    assert rc == A.OK, A.last_error()
    return d_vox.cpu().numpy()


def test_static_voxelizer_matches_prepare_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    specs = [ag.AirboxSpec(**SMALL), ag.random_spec(3, dx=4.0), ag.AirboxSpec(**SMALL), ag.config1_spec()]
    for n, spec in enumerate(specs):
        tris = ag.build_airbox(spec)
        g = E.prepare({"tris": tris, **spec.prepare_params()})
        want = g.fine()                                   # the allocating path
        got = static_voxelize(torch, local_triangles(g, tris), list(g.info.origin), g.h / 3,
                              3 * g.nx, 3 * g.ny, 3 * g.nz)
        assert got.shape == want.shape
        assert np.array_equal(got, want), f"call {n}: {int((got != want).sum())} voxels differ"


def test_static_voxelizer_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    d_tris = torch.zeros(9, dtype=torch.float32, device="cuda")
    d_vox = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = A.load().abx_voxelize_static(C.c_void_p(d_tris.data_ptr()), 9, (C.c_double * 3)(0.0, 0.0, 0.0), 1.0,
                                      4000, 4000, 2, C.c_void_p(d_vox.data_ptr()), None)
    assert rc == A.ERR_INVALID_ARGUMENT
    assert "scratch" in A.last_error()
    assert int(d_vox.sum().item()) == 0                # nothing was written
