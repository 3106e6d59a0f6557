"""Host mirror of the reference engine surface, src/engine.js
``module.exports = {parseSTL, makeFrame, prepare, setupSim, cpuStep, simulate, evaluate, ...}``
(src/engine.js:803), over libairbox.so.

Names, parameter objects and error messages follow engine.js, so code written
against the reference reads the same: ``prepare(p)`` takes the same ``p``
(tris, dx, sealAxis, sealSign, seal, inletAxis, inletSign, inletYaw, click,
pleat, outlet), ``simulate(g, p, onProgress, ns)`` takes the same run
parameters (K, aniso, u, tau, steps, avg, every) and returns the evaluate()
result object.  Errors the reference throws raise :class:`AirboxError` with
the reference's message text.

Every compute call runs on the GPU through the C ABI; there is no CPU path.
Extra keys: ``prepare`` accepts ``maxCells`` (the reference's cap is 4.5e6
cells, src/engine.js:124) and ``device``; ``simulate`` accepts ``storage``
("f32", "f32exact", "f16", "bf16", "f64").
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Callable, Optional

import numpy as np

from . import _abi as A


class AirboxError(RuntimeError):
    """An error of the engine; ``code`` is the abx_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def _check(rc: int):
    if rc != A.OK:
        raise AirboxError(rc, A.last_error())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------------------ parseSTL
def parseSTL(buf: bytes) -> np.ndarray:
    """parseSTL (src/engine.js:15-28): binary or ASCII STL -> float32 triangles (9 per triangle)."""
    L = A.load()
    n = C.c_size_t(0)
    buf = bytes(buf)
    _check(L.abx_parse_stl(buf, len(buf), None, 0, C.byref(n)))
    out = np.empty(n.value, np.float32)
    _check(L.abx_parse_stl(buf, len(buf), _ptr(out), out.size, C.byref(n)))
    return out


# ------------------------------------------------------------------------------ makeFrame
class Frame:
    """makeFrame (src/engine.js:31-43): local X (free axis), D (depth from the
    seal, into the box), Z (from the inlet side inwards), yawed about D."""

    def __init__(self, p: dict):
        dAx, iAx = p["sealAxis"], p["inletAxis"]
        if dAx == iAx:
            raise AirboxError(A.ERR_SAME_AXIS, "Einlassseite und Filterebene liegen auf derselben Achse.")
        self.dAx, self.iAx, self.oAx = dAx, iAx, 3 - dAx - iAx
        self.sd, self.si, self.seal = p["sealSign"], p["inletSign"], p["seal"]
        self.yaw = p.get("inletYaw") or 0
        yaw = self.yaw * math.pi / 180
        self.cy, self.sy = math.cos(yaw), math.sin(yaw)

    def toLocal(self, q):
        a, b = q[self.oAx], -self.si * q[self.iAx]
        return [self.cy * a + self.sy * b, -self.sd * (q[self.dAx] - self.seal), -self.sy * a + self.cy * b]

    def toModel(self, X, D, Z):
        q = [0.0, 0.0, 0.0]
        q[self.oAx] = self.cy * X - self.sy * Z
        q[self.dAx] = self.seal - self.sd * D
        q[self.iAx] = -self.si * (self.sy * X + self.cy * Z)
        return q

    def dirToModel(self, X, D, Z):
        q = [0.0, 0.0, 0.0]
        q[self.oAx] = self.cy * X - self.sy * Z
        q[self.dAx] = -self.sd * D
        q[self.iAx] = -self.si * (self.sy * X + self.cy * Z)
        return q


def makeFrame(p: dict) -> Frame:
    return Frame(p)


# ------------------------------------------------------------------------------ prepare
class Geometry:
    """The prepare() result (src/engine.js:226-233), device-resident.

    Scalars are read at once; each of the masks (solid, fluid, opening, outlet)
    and xc/dc/zc is copied to the host on its first access, on its own (the
    N-byte masks only when asked for)."""

    # abx_geom_get_masks argument order
    _ARRAYS = ("solid", "fluid", "opening", "outlet", "xc", "dc", "zc")

    def __init__(self, handle: C.c_void_p, p: dict):
        self._h = handle
        self.fr = Frame(p)
        info = A.GeomInfo()
        _check(A.load().abx_geom_get_info(handle, C.byref(info)))
        self.info = info
        self.h, self.nx, self.ny, self.nz, self.N = info.h, info.nx, info.ny, info.nz, int(info.N)
        self.top, self.jm, self.nf, self.pleat = info.top, info.jm, info.nf, info.pleat
        self.mn, self.mx = list(info.mn), list(info.mx)
        self.origin = list(info.origin)
        self._arrays = {}

    def _array(self, key: str) -> np.ndarray:
        a = self._arrays.get(key)
        if a is None:
            n, dt = {"solid": (self.N, np.uint8), "fluid": (self.N, np.uint8), "outlet": (self.N, np.uint8),
                     "opening": (self.nx * self.ny, np.uint8), "xc": (self.nx, np.float32),
                     "dc": (self.ny, np.float32), "zc": (self.nz, np.float32)}[key]
            a = np.empty(n, dt)
            _check(A.load().abx_geom_get_masks(self._h, *[_ptr(a) if k == key else None for k in self._ARRAYS]))
            self._arrays[key] = a
        return a

    solid = property(lambda self: self._array("solid"))
    fluid = property(lambda self: self._array("fluid"))
    opening = property(lambda self: self._array("opening"))
    outlet = property(lambda self: self._array("outlet"))
    xc = property(lambda self: self._array("xc"))
    dc = property(lambda self: self._array("dc"))
    zc = property(lambda self: self._array("zc"))

    def fine(self) -> np.ndarray:
        """voxelize()'s fine grid (3x per axis), recomputed on the GPU."""
        n = 27 * self.N
        out = np.empty(n, np.uint8)
        _check(A.load().abx_geom_get_fine(self._h, _ptr(out), n))
        return out

    @property
    def summary(self) -> dict:
        i = self.info
        s = {"grid": [self.nx, self.ny, self.nz], "cells": self.nf, "volume_l": i.volume_l,
             "inlet_cm2": i.inlet_cm2, "filter_cm2": i.filter_cm2, "outlet_cm2": i.outlet_cm2,
             "nHoles": i.n_holes, "outlet_cm2_real": i.outlet_cm2_real, "pleatOk": bool(i.pleat_ok)}
        # preview points in model coordinates (src/engine.js:218-224)
        xc, dc, zc, fl, op = self.xc, self.dc, self.zc, self.fluid, self.opening
        ny, nz = self.ny, self.nz
        fp = []
        lay = fl.reshape(self.nx, ny, nz)[:, self.jm, :]
        for ii, kk in zip(*np.nonzero(lay)):
            fp.extend(self.fr.toModel(float(xc[ii]), float(dc[self.jm]), float(zc[kk])))
        opn = []
        for c in np.nonzero(op)[0]:
            opn.extend(self.fr.toModel(float(xc[c // ny]), float(dc[c % ny]), self.mn[2]))
        s["openPts"], s["filterPts"] = opn, fp
        return s

    def __del__(self):
        try:
            if self._h:
                A.load().abx_geom_free(self._h)
                self._h = None
        except Exception:
            pass


def prepare(p: dict) -> Geometry:
    """prepare(p) (src/engine.js:111-234) on the GPU."""
    L = A.load()
    tris = np.ascontiguousarray(p["tris"], np.float32).ravel()
    pp = A.PrepareParams()
    pp.dx = p["dx"]; pp.seal_axis = p["sealAxis"]; pp.seal_sign = p["sealSign"]; pp.seal = p["seal"]
    pp.inlet_axis = p["inletAxis"]; pp.inlet_sign = p["inletSign"]; pp.inlet_yaw = p.get("inletYaw") or 0
    pp.pleat = p["pleat"]
    if p.get("click") is not None:
        pp.has_click = 1
        pp.click[:] = [float(v) for v in p["click"]]
    out = p.get("outlet")
    if out and out.get("enabled"):
        pp.has_outlet = 1
        pp.outlet_center[:] = [float(v) for v in out["center"]]
        pp.outlet_diameter, pp.outlet_height = out["diameter"], out["height"]
    pp.max_cells = p.get("maxCells", 4.5e6)
    pp.device = p.get("device", 0)
    h = C.c_void_p()
    _check(L.abx_prepare(_ptr(tris), tris.size, C.byref(pp), C.byref(h)))
    return Geometry(h, p)


# ------------------------------------------------------------------------------ setupSim / simulate
class Simulation:
    """setupSim(g, p) (src/engine.js:239-264) with its device state."""

    def __init__(self, g: Geometry, p: dict, ns: Optional[np.ndarray] = None):
        self.g = g
        self.p = dict(p)
        rp = A.RunParams(K=p["K"], aniso=p["aniso"], u=p["u"], tau=p["tau"], steps=int(p.get("steps", 0)),
                         avg=int(p.get("avg", 0)), every=int(p.get("every", 1) or 1),
                         storage=A.STORAGE[p.get("storage", "f32")],
                         flags=A.RUN_ALLOW_BF16 if p.get("allowBf16") else 0)
        self._ns = None if ns is None else np.ascontiguousarray(ns, np.float32)
        h = C.c_void_p()
        _check(A.load().abx_sim_create(g._h, C.byref(rp), _ptr(self._ns), C.byref(h)))
        self._h = h
        self.refresh()

    def refresh(self):
        info = A.SimInfo()
        _check(A.load().abx_sim_get_info(self._h, C.byref(info)))
        self.info = info
        self.NF, self.Ain, self.Af, self.sig = info.NF, info.Ain, info.Af, info.sig
        self.u0, self.tau0, self.aniso, self.cs2s = info.u0, info.tau0, info.aniso, info.cs2s
        return info

    def reset(self):
        _check(A.load().abx_sim_reset(self._h))

    def step(self, n: int = 1, accumulate: bool = False):
        _check(A.load().abx_sim_step(self._h, int(n), 1 if accumulate else 0))

    def run(self, onProgress: Optional[Callable] = None):
        cb = A.PROGRESS_FN(0)
        keep = None
        if onProgress is not None:
            def _cb(info, user):
                i = info.contents
                r = onProgress({"step": i.step, "steps": i.steps, "gamma": i.gamma, "massRatio": i.mass_ratio,
                                "elapsed": i.elapsed_s, "eta": i.eta_s, "mlups": i.mlups, "device": "GPU"})
                return 1 if r is False else 0
            keep = cb = A.PROGRESS_FN(_cb)
        _check(A.load().abx_sim_run(self._h, cb, None))
        del keep

    def get_f(self) -> np.ndarray:
        f = np.empty(19 * self.NF, np.float32)
        _check(A.load().abx_sim_get_f(self._h, _ptr(f)))
        return f

    def set_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, np.float32)
        assert f.size == 19 * self.NF
        _check(A.load().abx_sim_set_f(self._h, _ptr(f)))

    def clear_acc(self):
        """Start a new averaging window (populations kept)."""
        _check(A.load().abx_sim_clear_acc(self._h))

    def get_acc(self) -> np.ndarray:
        a = np.empty(4 * self.NF, np.float32)
        _check(A.load().abx_sim_get_acc(self._h, _ptr(a)))
        return a

    def evaluate(self) -> dict:
        m = A.Metrics()
        g = self.g
        fmap = np.empty(g.nx * g.nz, np.float32)
        cap = self.p.get("steps", 0) // max(self.p.get("every", 1), 1) + 2
        hist = np.zeros(3 * cap, np.float64)
        nh = C.c_int(0)
        _check(A.load().abx_sim_evaluate(self._h, C.byref(m), _ptr(fmap), _ptr(hist), cap, C.byref(nh)))
        metrics = {k: getattr(m, k) for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean",
                                              "zeta", "inlet_cm2", "filter_cm2")}
        fr = g.fr
        return {"metrics": metrics, "hist": hist[:3 * nh.value].reshape(-1, 3).tolist(), "fmap": fmap,
                "nx": g.nx, "ny": g.ny, "nz": g.nz, "xc": g.xc.tolist(), "zc": g.zc.tolist(), "dc": g.dc.tolist(),
                "pleat": g.pleat,
                "frame": {"dAx": fr.dAx, "iAx": fr.iAx, "oAx": fr.oAx, "sd": fr.sd, "si": fr.si, "seal": fr.seal,
                          "yaw": fr.yaw},
                "_detail": {k: getattr(m, k) for k in ("wm", "cm", "n", "cn", "pinN", "pbN", "jb")}}

    def field3d(self) -> dict:
        """field3d (src/engine.js:698-719): spd, pst, loss on the whole grid (NaN = no air)."""
        g = self.g
        out = [np.empty(g.N, np.float32) for _ in range(3)]
        i = A.Field3DInfo()
        _check(A.load().abx_sim_field3d(self._h, *(_ptr(o) for o in out), C.byref(i)))
        return {"nx": g.nx, "ny": g.ny, "nz": g.nz, "h": i.h, "x0": i.x0, "d0": i.d0, "z0": i.z0,
                "spd": out[0], "pst": out[1], "loss": out[2], "jm": i.jm, "top": i.top, "pleat": i.pleat,
                "kB": i.kB, "zIn": i.zIn, "_pin": i.pin, "_rhoRef": i.rho_ref}

    def planes(self) -> dict:
        """The cut planes of evaluate (src/engine.js:662-680): planInlet, planLow, lon."""
        g = self.g
        P, Q = g.nx * g.nz, g.nz * g.ny
        buf = np.empty(6 * P + 3 * Q, np.float32)
        i = A.PlanesInfo()
        _check(A.load().abx_sim_planes(self._h, _ptr(buf), C.byref(i)))

        def plan(o, depth):
            return {"speed": buf[o:o + P], "ua": buf[o + P:o + 2 * P], "ub": buf[o + 2 * P:o + 3 * P],
                    "n1": g.nx, "n2": g.nz, "depth": depth}
        lon = {"speed": buf[6 * P:6 * P + Q], "ua": buf[6 * P + Q:6 * P + 2 * Q], "ub": buf[6 * P + 2 * Q:],
               "n1": g.nz, "n2": g.ny, "x": i.x_lon}
        return {"planInlet": plan(0, i.depth_inlet), "planLow": plan(3 * P, i.depth_low), "lon": lon,
                "_ic": i.ic, "_jc": i.jc, "_jlow": i.jlow}

    def streamlines(self, maxSeeds: int = 220) -> dict:
        """streamlines (src/engine.js:721-758), traced on the GPU: pts (model coordinates), spd, off."""
        i = A.LinesInfo()
        # capacities that always suffice: one call traces once
        cap = (maxSeeds + 1) * A.MAX_LINE_POINTS
        pts = np.empty(3 * cap, np.float32)
        spd = np.empty(cap, np.float32)
        off = np.empty(maxSeeds + 2, np.uint32)
        _check(A.load().abx_sim_streamlines(self._h, maxSeeds, _ptr(pts), _ptr(spd), _ptr(off), cap, maxSeeds + 2,
                                            C.byref(i)))
        return {"pts": pts[:3 * i.n_points], "spd": spd[:i.n_points], "off": off[:i.n_lines + 1]}

    def set_timing(self, on: bool = True):
        _check(A.load().abx_sim_set_timing(self._h, 1 if on else 0))

    def timing(self) -> dict:
        t = A.Timing()
        _check(A.load().abx_sim_get_timing(self._h, C.byref(t)))
        return {k: (float(getattr(t, k)) if isinstance(getattr(t, k), float) else int(getattr(t, k)))
                for k, _ in A.Timing._fields_}

    def __del__(self):
        try:
            if self._h:
                A.load().abx_sim_free(self._h)
                self._h = None
        except Exception:
            pass


def setupSim(g: Geometry, p: dict, ns=None) -> Simulation:
    return Simulation(g, p, ns)


def cpuStep(S: Simulation, n: int = 1, accumulate: bool = False):
    """The reference's cpuStep (src/engine.js:266-321), n times, on the GPU."""
    S.step(n, accumulate)


def simulate(g: Geometry, p: dict, onProgress: Optional[Callable] = None, ns=None, full: bool = True) -> dict:
    """simulate(g, p, onProgress, ns) (src/engine.js:341-358): the step loop and evaluate().
    With full=False only the KPIs, filter map and history are read back (no planes, field3d, lines)."""
    if g is None:
        raise AirboxError(A.ERR_NOT_PREPARED, "Bitte zuerst die Geometrie prüfen.")
    S = Simulation(g, p, ns)
    S.run(onProgress)
    res = evaluate(S) if full else S.evaluate()
    res["device"] = "GPU"
    return res


def evaluate(S: Simulation) -> dict:
    """evaluate() (src/engine.js:632-691) of a finished simulation: KPIs, filter map, history, the cut
    planes (planInlet, planLow, lon), the 3-D fields (vol, field3d :698-719) and the streamlines (lines)."""
    res = S.evaluate()
    pl = S.planes()
    res.update({k: pl[k] for k in ("planInlet", "planLow", "lon")})
    res["vol"] = S.field3d()
    res["lines"] = S.streamlines()
    return res
