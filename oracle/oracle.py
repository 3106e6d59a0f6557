"""ORACLE ONLY - ctypes harness over oracle/_build/libengine_ref.so.

Test infrastructure: only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg import this module.  It wraps the plain-C restatement of the
reference compute core (src/engine.js: parseSTL, makeFrame, prepare,
setupSim, cpuStep, simulate, evaluate) that engine_ref.c implements.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libengine_ref.so")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = [os.path.join(HERE, f) for f in ("engine_ref.c", "engine_ref_post.c", "engine_ref_step.inc", "engine_ref.h")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class Frame(C.Structure):
    _fields_ = [("dAx", C.c_int), ("iAx", C.c_int), ("oAx", C.c_int),
                ("sd", C.c_double), ("si", C.c_double), ("seal", C.c_double),
                ("yaw_deg", C.c_double), ("cy", C.c_double), ("sy", C.c_double)]


class PrepParams(C.Structure):
    _fields_ = [("dx", C.c_double), ("sealAxis", C.c_int), ("sealSign", C.c_double), ("seal", C.c_double),
                ("inletAxis", C.c_int), ("inletSign", C.c_double), ("inletYaw", C.c_double),
                ("pleat", C.c_double), ("has_click", C.c_int), ("click", C.c_double * 3),
                ("has_outlet", C.c_int), ("out_center", C.c_double * 3), ("out_diameter", C.c_double),
                ("out_height", C.c_double), ("max_cells", C.c_double), ("keep_fine", C.c_int)]


class Geom(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("N", C.c_int64),
                ("nxf", C.c_int), ("nyf", C.c_int), ("nzf", C.c_int), ("kf", C.c_int), ("kw0", C.c_int),
                ("h", C.c_double), ("hf", C.c_double), ("origin", C.c_double * 3), ("mn", C.c_double * 3),
                ("mx", C.c_double * 3), ("pleat", C.c_double),
                ("top", C.c_int), ("jm", C.c_int), ("nf", C.c_int), ("nOpen", C.c_int), ("Af", C.c_int),
                ("nHoles", C.c_int), ("nOut", C.c_int), ("leak", C.c_int), ("jpt", C.c_int),
                ("fr", Frame),
                ("xc", C.POINTER(C.c_float)), ("dc", C.POINTER(C.c_float)), ("zc", C.POINTER(C.c_float)),
                ("solid", C.POINTER(C.c_uint8)), ("fluid", C.POINTER(C.c_uint8)),
                ("opening", C.POINTER(C.c_uint8)), ("outlet", C.POINTER(C.c_uint8)),
                ("fine", C.POINTER(C.c_uint8)), ("holes_slice", C.POINTER(C.c_uint8)),
                ("err", C.c_int), ("msg", C.c_char * 512)]


class RunParams(C.Structure):
    _fields_ = [("K", C.c_double), ("aniso", C.c_double), ("u", C.c_double), ("tau", C.c_double)]


class Sim(C.Structure):
    _fields_ = [("NF", C.c_int), ("Ain", C.c_int), ("Af", C.c_int), ("Lp", C.c_int), ("nM", C.c_int), ("nT", C.c_int),
                ("u0", C.c_double), ("tau0", C.c_double), ("sig", C.c_double), ("aniso", C.c_double),
                ("cs2s", C.c_double),
                ("cid", C.POINTER(C.c_int32)), ("cells", C.POINTER(C.c_int32)), ("nb", C.POINTER(C.c_int32)),
                ("jsOf", C.POINTER(C.c_int32)), ("layerM", C.POINTER(C.c_int32)), ("layerT", C.POINTER(C.c_int32)),
                ("flag", C.POINTER(C.c_uint32)), ("N", C.c_int64)]


class Metrics(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean",
                                          "zeta", "inlet_cm2", "filter_cm2", "wm", "cm")] + \
               [(k, C.c_int) for k in ("n", "cn", "pinN", "pbN", "jb")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        fp = C.c_void_p
        L.ora_parse_stl.argtypes = [C.c_char_p, C.c_size_t, fp, C.c_size_t, C.POINTER(C.c_size_t), C.c_char_p]
        L.ora_prepare.argtypes = [fp, C.c_size_t, C.POINTER(PrepParams), C.POINTER(Geom)]
        L.ora_geom_free.argtypes = [C.POINTER(Geom)]
        L.ora_voxelize.argtypes = [fp, C.c_size_t, C.c_double * 3, C.c_int, C.c_int, C.c_int, C.c_double, fp]
        L.ora_setup.argtypes = [C.POINTER(Geom), C.POINTER(RunParams), C.POINTER(Sim)]
        L.ora_sim_free.argtypes = [C.POINTER(Sim)]
        L.ora_to_local.argtypes = [C.POINTER(Frame), C.c_double * 3, C.c_double * 3]
        L.ora_make_frame.argtypes = [C.POINTER(PrepParams), C.POINTER(Frame)]
        for nm in ("ora_init_f32", "ora_init_f64"):
            getattr(L, nm).argtypes = [C.POINTER(Sim), fp]
        for nm in ("ora_step_f32", "ora_step_f64", "ora_step_f32l"):
            getattr(L, nm).argtypes = [C.POINTER(Sim), fp, fp, fp, fp, C.c_int]
        for nm in ("ora_simulate_f32", "ora_simulate_f64"):
            getattr(L, nm).argtypes = [C.POINTER(Sim), C.c_int, C.c_int, C.c_int, fp, C.c_int, fp, fp,
                                       C.POINTER(C.c_int), C.c_char_p]
        for nm in ("ora_evaluate_f32", "ora_evaluate_f64"):
            getattr(L, nm).argtypes = [C.POINTER(Geom), C.POINTER(Sim), C.c_double, fp, fp, C.POINTER(Metrics), fp]
        L.ora_js_hypot3.restype = C.c_double
        L.ora_js_hypot3.argtypes = [C.c_double] * 3
        L.ora_field3d.argtypes = [C.POINTER(Geom), C.POINTER(Sim), C.c_double, fp, fp, fp, fp, fp,
                                  C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.ora_planes.argtypes = [C.POINTER(Geom), C.POINTER(Sim), C.c_double, fp, fp, fp, C.c_int * 3]
        L.ora_streamlines.argtypes = [C.POINTER(Geom), C.POINTER(Sim), C.c_double, fp, fp, C.c_int, fp, fp, fp,
                                      C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def parse_stl(buf: bytes) -> np.ndarray:
    n = C.c_size_t(0)
    msg = C.create_string_buffer(512)
    rc = lib().ora_parse_stl(buf, len(buf), None, 0, C.byref(n), msg)
    if rc:
        raise OracleError(rc, msg.value.decode())
    out = np.empty(n.value, np.float32)
    rc = lib().ora_parse_stl(buf, len(buf), _ptr(out), out.size, C.byref(n), msg)
    if rc:
        raise OracleError(rc, msg.value.decode())
    return out


def prep_params(p: dict, max_cells: float = 4.5e6, keep_fine: bool = False) -> PrepParams:
    pp = PrepParams()
    pp.dx = p["dx"]; pp.sealAxis = p["sealAxis"]; pp.sealSign = p["sealSign"]; pp.seal = p["seal"]
    pp.inletAxis = p["inletAxis"]; pp.inletSign = p["inletSign"]; pp.inletYaw = p.get("inletYaw", 0) or 0
    pp.pleat = p["pleat"]
    if p.get("click") is not None:
        pp.has_click = 1
        pp.click[:] = list(p["click"])
    out = p.get("outlet")
    if out and out.get("enabled"):
        pp.has_outlet = 1
        pp.out_center[:] = list(out["center"])
        pp.out_diameter = out["diameter"]; pp.out_height = out["height"]
    pp.max_cells = max_cells
    pp.keep_fine = 1 if keep_fine else 0
    return pp


@dataclass
class OracleGeom:
    g: Geom
    nx: int
    ny: int
    nz: int

    def arr(self, name, n, dtype=np.uint8):
        p = getattr(self.g, name)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dtype, copy=True)

    @property
    def N(self):
        return self.nx * self.ny * self.nz

    def solid(self): return self.arr("solid", self.N)
    def fluid(self): return self.arr("fluid", self.N)
    def outlet(self): return self.arr("outlet", self.N)
    def opening(self): return self.arr("opening", self.nx * self.ny)
    def fine(self): return self.arr("fine", self.g.nxf * self.g.nyf * self.g.nzf)
    def holes_slice(self): return self.arr("holes_slice", self.g.nxf * self.g.nyf)
    def dc(self): return self.arr("dc", self.ny, np.float32)
    def xc(self): return self.arr("xc", self.nx, np.float32)
    def zc(self): return self.arr("zc", self.nz, np.float32)

    def __del__(self):
        try:
            lib().ora_geom_free(C.byref(self.g))
        except Exception:
            pass


def prepare(tris: np.ndarray, p: dict, max_cells: float = 4.5e6, keep_fine: bool = False) -> OracleGeom:
    tris = np.ascontiguousarray(tris, np.float32).ravel()
    g = Geom()
    pp = prep_params(p, max_cells, keep_fine)
    rc = lib().ora_prepare(_ptr(tris), tris.size, C.byref(pp), C.byref(g))
    if rc:
        msg = g.msg.decode()
        lib().ora_geom_free(C.byref(g))
        raise OracleError(rc, msg)
    return OracleGeom(g, g.nx, g.ny, g.nz)


def voxelize(tris, origin, nx, ny, nz, h) -> np.ndarray:
    tris = np.ascontiguousarray(tris, np.float32).ravel()
    out = np.zeros(nx * ny * nz, np.uint8)
    lib().ora_voxelize(_ptr(tris), tris.size, (C.c_double * 3)(*origin), nx, ny, nz, h, _ptr(out))
    return out.reshape(nx, ny, nz)


class OracleSim:
    """setupSim (src/engine.js:239-264) plus step/simulate/evaluate."""

    def __init__(self, og: OracleGeom, run: dict):
        self.og = og
        self.S = Sim()
        rp = RunParams(K=run["K"], aniso=run["aniso"], u=run["u"], tau=run["tau"])
        lib().ora_setup(C.byref(og.g), C.byref(rp), C.byref(self.S))
        self.u0 = run["u"]
        self.NF = self.S.NF

    def __del__(self):
        try:
            lib().ora_sim_free(C.byref(self.S))
        except Exception:
            pass

    def cells(self): return np.ctypeslib.as_array(self.S.cells, shape=(self.NF,)).copy()
    def nb(self): return np.ctypeslib.as_array(self.S.nb, shape=(self.NF * 19,)).copy()
    def flag(self): return np.ctypeslib.as_array(self.S.flag, shape=(self.NF,)).copy()
    def layerM(self): return np.ctypeslib.as_array(self.S.layerM, shape=(self.S.nM,)).copy()
    def layerT(self): return np.ctypeslib.as_array(self.S.layerT, shape=(self.S.nT,)).copy()

    def f0(self, dtype=np.float32):
        f = np.empty(19 * self.NF, dtype)
        (lib().ora_init_f32 if dtype == np.float32 else lib().ora_init_f64)(C.byref(self.S), _ptr(f))
        return f

    def step(self, f, acc=None, ns=None, kind="f32", nthreads=0):
        f2 = np.empty_like(f)
        fn = {"f32": lib().ora_step_f32, "f64": lib().ora_step_f64, "f32l": lib().ora_step_f32l}[kind]
        fn(C.byref(self.S), _ptr(f), _ptr(f2), _ptr(acc), _ptr(ns), nthreads or os.cpu_count())
        return f2

    def simulate(self, steps, avg, every, ns=None, kind="f32", nthreads=0):
        dt = np.float32 if kind == "f32" else np.float64
        acc = np.empty(4 * self.NF, dt)
        hist = np.zeros(3 * (steps // max(every, 1) + 2), np.float64)
        nh = C.c_int(0)
        msg = C.create_string_buffer(512)
        fn = lib().ora_simulate_f32 if kind == "f32" else lib().ora_simulate_f64
        rc = fn(C.byref(self.S), steps, avg, every, _ptr(ns), nthreads or os.cpu_count(), _ptr(acc), _ptr(hist),
                C.byref(nh), msg)
        if rc:
            raise OracleError(rc, msg.value.decode())
        return acc, hist[:3 * nh.value].reshape(-1, 3)

    def field3d(self, acc, ns=None):
        """field3d (src/engine.js:698-719) of float32 averages: spd, pst, loss (nx, ny, nz) and kB, pin, rhoRef."""
        N = self.og.nx * self.og.ny * self.og.nz
        out = [np.empty(N, np.float32) for _ in range(3)]
        kB, pin, rr = C.c_int(), C.c_double(), C.c_double()
        lib().ora_field3d(C.byref(self.og.g), C.byref(self.S), self.u0, _ptr(acc), _ptr(ns), *(_ptr(o) for o in out),
                          C.byref(kB), C.byref(pin), C.byref(rr))
        sh = (self.og.nx, self.og.ny, self.og.nz)
        return [o.reshape(sh) for o in out], kB.value, pin.value, rr.value

    def planes(self, acc, ns=None):
        """evaluate's cut planes (src/engine.js:662-680): one float32 buffer and (ic, jc, jlow)."""
        nx, ny, nz = self.og.nx, self.og.ny, self.og.nz
        out = np.empty(6 * nx * nz + 3 * nz * ny, np.float32)
        meta = (C.c_int * 3)()
        lib().ora_planes(C.byref(self.og.g), C.byref(self.S), self.u0, _ptr(acc), _ptr(ns), _ptr(out), meta)
        return out, tuple(meta)

    def streamlines(self, acc, ns=None, max_seeds=220):
        """streamlines (src/engine.js:721-758): pts (model coordinates), spd, off."""
        cap_pts, cap_lines = 2100 * max(max_seeds, 1), max_seeds + 2
        pts = np.empty(3 * cap_pts, np.float32)
        spd = np.empty(cap_pts, np.float32)
        off = np.empty(cap_lines, np.uint32)
        nl, npt = C.c_int(), C.c_int()
        rc = lib().ora_streamlines(C.byref(self.og.g), C.byref(self.S), self.u0, _ptr(acc), _ptr(ns), max_seeds,
                                   _ptr(pts), _ptr(spd), _ptr(off), cap_pts, cap_lines, C.byref(nl), C.byref(npt))
        assert rc == 0
        return pts[:3 * npt.value], spd[:npt.value], off[:nl.value + 1]

    def evaluate(self, acc, ns=None):
        m = Metrics()
        fmap = np.empty(self.og.nx * self.og.nz, np.float32)
        fn = lib().ora_evaluate_f32 if acc.dtype == np.float32 else lib().ora_evaluate_f64
        fn(C.byref(self.og.g), C.byref(self.S), self.u0, _ptr(acc), _ptr(ns), C.byref(m), _ptr(fmap))
        out = {k: getattr(m, k) for k, _ in Metrics._fields_}
        return out, fmap.reshape(self.og.nx, self.og.nz)
