"""libairbox.so loads, exports every entry point include/airbox.h declares,
and its host-only STL parser agrees with the oracle (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from airboxcalc_gb300 import _abi as A
from airboxcalc_gb300 import airboxgen as ag
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "airbox_cfd_golden.npz"))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "airbox.h")).read()
    return sorted(set(re.findall(r"\b(abx_[a-z_0-9]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert header_symbols() == sorted(A.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = A.load()
    for name in header_symbols():
        assert hasattr(L, name), name
    assert L.abx_abi_version() == A.ABI_VERSION == 3


@pytest.mark.parametrize("key", ["stl_binary", "stl_ascii"])
def test_parse_stl_matches_oracle_and_reference(key):
    from airboxcalc_gb300 import engine as E
    buf = GOLD[key].tobytes()
    got = E.parseSTL(buf)
    assert np.array_equal(got, O.parse_stl(buf))
    assert np.array_equal(got, GOLD[key + "_parsed"])


def test_parse_stl_errors():
    from airboxcalc_gb300 import engine as E
    with pytest.raises(E.AirboxError) as ei:
        E.parseSTL(b"solid nothing\nendsolid\n")
    assert ei.value.code == A.ERR_NO_TRIANGLES and "keine Dreiecke" in str(ei.value)
    weird = b"vertex 1.2.3 0 0 vertex 1 0 0 vertex 0 1 0 vertex 9 9\nvertex 1 2 3"
    a, b = E.parseSTL(weird), O.parse_stl(weird)
    assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_binary_stl_of_generated_airbox_roundtrips():
    from airboxcalc_gb300 import engine as E
    tris = ag.build_airbox(ag.random_spec(3, dx=3.0))
    assert np.array_equal(E.parseSTL(ag.to_binary_stl(tris)), tris.ravel())


def test_compute_calls_fail_loudly_without_gpu():
    from airboxcalc_gb300 import engine as E
    if A.load().abx_device_count() > 0:
        pytest.skip("a GPU is visible")
    spec = ag.config1_spec()
    with pytest.raises(E.AirboxError) as ei:
        E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params()})
    assert ei.value.code == A.ERR_CUDA


def test_warm_start_and_batch_entry_points_check_arguments_without_gpu():
    """Argument checks answer before any CUDA call; valid calls fail loudly (no CPU fallback)."""
    import ctypes as C
    L = A.load()
    h = C.c_void_p()
    bad = A.NetParams(res=12, base=16, levels=4, device=0, seed=0)
    assert L.abx_net_create(C.byref(bad), C.byref(h)) == A.ERR_INVALID_ARGUMENT
    assert "power of two" in A.last_error()
    bad = A.NetParams(res=64, base=12, levels=4, device=0, seed=0)
    assert L.abx_net_create(C.byref(bad), C.byref(h)) == A.ERR_INVALID_ARGUMENT
    ok = A.NetParams(res=64, base=16, levels=4, device=0, seed=0)
    assert L.abx_net_create(C.byref(ok), C.byref(h)) == A.ERR_CUDA          # no GPU here
    r = A.ConvergeResult()
    assert L.abx_sim_converge(None, None, C.byref(r)) == A.ERR_INVALID_ARGUMENT
    assert L.abx_batch_create(None, None, 0, C.byref(h)) == A.ERR_INVALID_ARGUMENT
    assert L.abx_sim_streamlines(None, 220, None, None, None, 0, 0, None) == A.ERR_INVALID_ARGUMENT


def test_prepare_rejects_grids_beyond_32_bit_offsets_before_any_gpu_work():
    """The step kernels index populations with 32-bit offsets: 19 * padded cells must stay below 2^32."""
    from airboxcalc_gb300 import engine as E
    tris = np.array([[0, 0, 0], [3000, 0, 0], [0, 3000, 0], [0, 0, 0], [0, 0, 3000], [3000, 0, 0]],
                    np.float32).ravel()
    p = {"tris": tris, "dx": 1.0, "sealAxis": 1, "sealSign": -1, "seal": 0, "inletAxis": 2, "inletSign": -1,
         "inletYaw": 0, "pleat": 40, "maxCells": 1e12}
    with pytest.raises(E.AirboxError) as ei:
        E.prepare(p)
    assert ei.value.code == A.ERR_INVALID_ARGUMENT and "2^32" in str(ei.value)
    with pytest.raises(E.AirboxError) as ei:
        E.prepare({**p, "maxCells": 4.5e6})               # the reference's own cap comes first
    assert ei.value.code == A.ERR_GRID_TOO_LARGE and "Gitter zu groß" in str(ei.value)


def test_geometry_copies_each_array_on_its_own(monkeypatch):
    """The Python Geometry asks abx_geom_get_masks for one array per call, on first access only: reading the
    coordinates (as evaluate() does) never copies the N-byte masks."""
    from airboxcalc_gb300 import engine as E
    calls = []

    class FakeLib:
        def abx_geom_get_masks(self, h, *ptrs):
            asked = [k for k, p in zip(E.Geometry._ARRAYS, ptrs) if p is not None]
            calls.append(asked)
            return A.OK

    monkeypatch.setattr(A, "load", lambda *a, **k: FakeLib())
    g = object.__new__(E.Geometry)
    g._h, g.N, g.nx, g.ny, g.nz, g._arrays = C.c_void_p(1), 6 * 5 * 4, 6, 5, 4, {}
    assert g.xc.shape == (6,) and g.zc.shape == (4,) and g.dc.shape == (5,)
    assert g.xc is g.xc and g.opening.shape == (30,)
    assert calls == [["xc"], ["zc"], ["dc"], ["opening"]]
    assert g.fluid.shape == (120,) and g.fluid.dtype == np.uint8
    assert calls[-1] == ["fluid"] and len(calls) == 5
    g._h = None                      # a stand-in handle: nothing to free
