"""Learned warm start: the network, its training on fields the LBM produces,
and the windowed convergence run (Python side of the C ABI's abx_net_* /
abx_sim_warm_start / abx_sim_converge / abx_sim_solve_warm).

The reference has no counterpart: engine.js starts every run from f = w_i
(src/engine.js:261) and runs the fixed steps/avg schedule (:341-358).  Here a
3-D convolutional encoder-decoder predicts the time-averaged velocity and
density from the voxelized geometry; the solve starts from their equilibrium,
settles, then grows a running average until its gamma core and zeta stop
moving, and falls back to the uniform start and the full schedule when they
do not.  Training, inference and the initialisation run in the library's CUDA
kernels; this module only moves parameters and drives the loop.

Command line (trains on the GPU and writes the weights; the defaults are the
shipped network's recipe: 4000 seeded airboxes at dx 2 mm, 100 epochs):
    python -m airboxcalc_gb300.warmstart --out weights.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import sys
import time
from typing import Optional

import numpy as np

from . import _abi as A
from . import airboxgen as ag
from . import engine as E

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "warmstart_r64_b16_l4.npz")
# The reference's run parameters (the fixed schedule the plain solve follows).
RUN = dict(K=3, aniso=10, u=0.06, tau=0.51, steps=6000, avg=2000, every=150)
K_CHOICES = (1.5, 3.0, 6.0)
# Stop rule of the convergence run: settle, then a running average checked every window.
CONVERGE = dict(settle=1000, window=500, min_avg=1000, max_steps=4000, tol=0.01, rule=0, min_windows=4)


def variant(seed: int, dx: float = 2.0):
    """Airbox `seed` of the seeded generator at cell size dx and its filter K."""
    return ag.random_spec(seed, dx=dx), K_CHOICES[seed % 3]


class Net:
    """The warm-start network on one GPU (abx_net)."""

    def __init__(self, res: int = 64, base: int = 16, levels: int = 4, device: int = 0, seed: int = 0,
                 coords: bool = False):
        p = A.NetParams(res=res, base=base, levels=levels, device=device, seed=seed, coords=1 if coords else 0)
        h = C.c_void_p()
        E._check(A.load().abx_net_create(C.byref(p), C.byref(h)))
        self._h = h
        self.res, self.base, self.levels, self.coords = res, base, levels, bool(coords)
        self.V = res ** 3
        self.n_in = 12 if coords else 9

    @property
    def info(self) -> dict:
        i = A.NetInfo()
        E._check(A.load().abx_net_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in A.NetInfo._fields_}

    def set_tensor_cores(self, on: bool = True):
        """Convolutions on the tensor cores (tcgen05, bf16 operands) or on the float32 kernels."""
        E._check(A.load().abx_net_set_tensor_cores(self._h, 1 if on else 0))

    @property
    def n_params(self) -> int:
        return self.info["n_params"]

    def get_weights(self) -> np.ndarray:
        w = np.empty(self.n_params, np.float32)
        E._check(A.load().abx_net_get_weights(self._h, E._ptr(w)))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        if w.size != self.n_params:
            raise ValueError(f"expected {self.n_params} weights, got {w.size}")
        E._check(A.load().abx_net_set_weights(self._h, E._ptr(w)))

    def save(self, path: str, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, weights=self.get_weights(), res=self.res, base=self.base, levels=self.levels,
                            coords=int(self.coords), meta=json.dumps(meta))

    @classmethod
    def load(cls, path: str = WEIGHTS, device: int = 0) -> "Net":
        d = np.load(path)
        n = cls(int(d["res"]), int(d["base"]), int(d["levels"]), device=device,
                coords=bool(int(d["coords"])) if "coords" in d else False)
        n.set_weights(d["weights"])
        n.meta = json.loads(str(d["meta"])) if "meta" in d else {}
        return n

    def add_sample(self, sim: E.Simulation):
        E._check(A.load().abx_net_add_sample(self._h, sim._h))

    def clear_samples(self):
        E._check(A.load().abx_net_clear_samples(self._h))

    def sample(self, i: int):
        V = self.V
        x = np.empty(self.n_in * V, np.float32)
        t = np.empty(4 * V, np.float32)
        m = np.empty(V, np.float32)
        E._check(A.load().abx_net_get_sample(self._h, i, E._ptr(x), E._ptr(t), E._ptr(m)))
        r = self.res
        return x.reshape(self.n_in, r, r, r), t.reshape(4, r, r, r), m.reshape(r, r, r)

    def train(self, first: int, count: int, epochs: int, batch: int = 8, lr: float = 1e-3, lr_min: float = 1e-5,
              seed: int = 0, flip: bool = True) -> np.ndarray:
        p = A.TrainParams(first=first, count=count, epochs=epochs, batch=batch, lr=lr, lr_min=lr_min, seed=seed,
                          flip=1 if flip else 0)
        out = np.zeros(epochs, np.float64)
        E._check(A.load().abx_net_train(self._h, C.byref(p), E._ptr(out)))
        return out

    def eval_loss(self, first: int, count: int) -> float:
        v = C.c_double()
        E._check(A.load().abx_net_eval_loss(self._h, first, count, C.byref(v)))
        return v.value

    def forward_backward(self, d_x: int, d_t: int, d_m: int, B: int, scale: float, d_pred: int,
                         d_grad: Optional[int]) -> float:
        """One pass on caller device buffers (raw pointers); returns the loss."""
        v = C.c_double()
        E._check(A.load().abx_net_forward_backward(self._h, C.c_void_p(d_x), C.c_void_p(d_t), C.c_void_p(d_m), B,
                                                   scale, C.c_void_p(d_pred),
                                                   C.c_void_p(d_grad) if d_grad else None, C.byref(v)))
        return v.value

    def predict(self, sim: E.Simulation):
        r = self.res
        x = np.empty(self.n_in * self.V, np.float32)
        y = np.empty(4 * self.V, np.float32)
        E._check(A.load().abx_net_predict(self._h, sim._h, E._ptr(x), E._ptr(y)))
        return x.reshape(self.n_in, r, r, r), y.reshape(4, r, r, r)

    def __del__(self):
        try:
            if self._h:
                A.load().abx_net_free(self._h)
                self._h = None
        except Exception:
            pass


def _metrics(m: A.Metrics) -> dict:
    return {k: getattr(m, k) for k in ("gamma", "gammaCore", "lowCore", "highCore", "reverse", "maxToMean", "zeta")}


def _converge_params(**kw) -> A.ConvergeParams:
    c = dict(CONVERGE, **kw)
    return A.ConvergeParams(settle=int(c["settle"]), window=int(c["window"]), min_avg=int(c["min_avg"]),
                            max_steps=int(c["max_steps"]), tol=float(c["tol"]), rule=int(c["rule"]),
                            min_windows=int(c["min_windows"]))


def warm_start(sim: E.Simulation, net: Net):
    """f = feq of the network's prediction on every fluid cell."""
    E._check(A.load().abx_sim_warm_start(sim._h, net._h))


def converge(sim: E.Simulation, **kw) -> dict:
    """Settle, then a running average until its KPIs stop moving (abx_sim_converge)."""
    r = A.ConvergeResult()
    E._check(A.load().abx_sim_converge(sim._h, C.byref(_converge_params(**kw)), C.byref(r)))
    return {"metrics": _metrics(r.metrics), "steps": r.steps, "windows": r.windows, "converged": bool(r.converged),
            "change": r.change}


def solve_warm(sim: E.Simulation, net: Net, **kw) -> dict:
    """Warm start, windowed run and fallback to the full schedule (abx_sim_solve_warm)."""
    r = A.WarmResult()
    E._check(A.load().abx_sim_solve_warm(sim._h, net._h, C.byref(_converge_params(**kw)), C.byref(r)))
    return {"metrics": _metrics(r.run.metrics), "steps": r.run.steps, "windows": r.run.windows,
            "converged": bool(r.run.converged), "change": r.run.change, "fell_back": bool(r.fell_back),
            "warm_steps": r.warm_steps, "infer_ms": r.infer_ms, "total_ms": r.total_ms}


def generate(net: Net, seeds, dx: float = 2.0, run: dict = RUN, log=None) -> list:
    """Training data: for each seed, the plain float32 solve on the fixed schedule; its time averages
    become one stored sample.  Returns one row (seed, grid, KPIs, times) per sample."""
    rows = []
    for seed in seeds:
        spec, K = variant(seed, dx)
        t0 = time.perf_counter()
        try:
            g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
            t1 = time.perf_counter()
            S = E.Simulation(g, dict(run, K=K))
            S.run()
        except E.AirboxError as e:   # leaking or unstable variants give no sample
            row = {"seed": seed, "K": K, "skipped": e.code, "message": str(e)}
            rows.append(row)
            if log:
                log(row)
            continue
        m = S.evaluate()["metrics"]
        net.add_sample(S)
        t2 = time.perf_counter()
        row = {"seed": seed, "K": K, "nx": g.nx, "ny": g.ny, "nz": g.nz, "NF": S.NF,
               "gammaCore": m["gammaCore"], "zeta": m["zeta"], "prepare_s": round(t1 - t0, 4),
               "solve_s": round(t2 - t1, 4)}
        rows.append(row)
        if log:
            log(row)
        del S, g
    return rows


def _range(s: str):
    a, b = s.split(":")
    return range(int(a), int(b))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train", default="0:4000", help="seed range a:b of the training airboxes")
    ap.add_argument("--val", default="5000:5064", help="seed range of the validation airboxes (loss only)")
    ap.add_argument("--dx", type=float, default=2.0)
    ap.add_argument("--res", type=int, default=64)
    ap.add_argument("--base", type=int, default=16)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--coords", action="store_true", help="add the voxel coordinates as input channels")
    ap.add_argument("--epochs", type=int, default=100)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-min", type=float, default=1e-5)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--log", default=None, help="JSON-lines log of the generated samples")
    a = ap.parse_args(argv)
    net = Net(a.res, a.base, a.levels, seed=a.seed, coords=a.coords)
    logf = open(a.log, "w") if a.log else None
    t0 = time.perf_counter()

    def log(row):
        if logf:
            logf.write(json.dumps(row) + "\n")
            logf.flush()

    rows_t = generate(net, _range(a.train), a.dx, log=log)
    rows_v = generate(net, _range(a.val), a.dx, log=log)
    t1 = time.perf_counter()
    nt = sum("skipped" not in r for r in rows_t)
    nv = sum("skipped" not in r for r in rows_v)
    print(json.dumps({"generated": nt + nv, "skipped": len(rows_t) + len(rows_v) - nt - nv,
                      "seconds": round(t1 - t0, 1)}), flush=True)
    v0 = net.eval_loss(nt, nv)
    hist = []
    for ep in range(a.epochs):
        # one epoch per call, so that the validation loss can be followed; each call decays the rate
        # from lr0 to lr1, which chains into one cosine schedule over the whole run
        frac0, frac1 = ep / a.epochs, (ep + 1) / a.epochs
        lr0 = a.lr_min + 0.5 * (a.lr - a.lr_min) * (1 + np.cos(np.pi * frac0))
        lr1 = a.lr_min + 0.5 * (a.lr - a.lr_min) * (1 + np.cos(np.pi * frac1))
        tl = net.train(0, nt, 1, a.batch, lr=lr0, lr_min=lr1, seed=a.seed * 1000 + ep, flip=True)[0]
        vl = net.eval_loss(nt, nv)
        hist.append([ep + 1, float(tl), float(vl)])
        print(json.dumps({"epoch": ep + 1, "train_loss": tl, "val_loss": vl,
                          "seconds": round(time.perf_counter() - t1, 1)}), flush=True)
    net.save(a.out, train=a.train, val=a.val, dx=a.dx, epochs=a.epochs, batch=a.batch, lr=a.lr, val_loss0=v0,
             history=hist)
    print(json.dumps({"saved": a.out, "n_params": net.n_params, "val_loss_untrained": v0,
                      "val_loss": hist[-1][2] if hist else v0}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
