"""Batched variants: many airboxes of uneven size advanced together, one
kernel launch per LBM step over all of them (abx_batch_* of the C ABI).

The reference batches only variants that share one geometry (GpuSim,
src/engine.js:495-545: B copies of the populations stepped by one lbm_step
dispatch, for filter/ns variants of one airbox); here every variant has its
own geometry, K, aniso, u and tau.  The block shape of the batched step
kernel is chosen by an autotuner that times the candidates on the batch's
own domains.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _abi as A
from . import engine as E


class BatchVariant(E.Simulation):
    """A variant of a batch seen as a simulation (evaluate, get_acc, get_f); owned by the batch."""

    def __init__(self, batch: "Batch", i: int, g: E.Geometry, p: dict):
        h = C.c_void_p()
        E._check(A.load().abx_batch_sim(batch._h, i, C.byref(h)))
        self._h, self.g, self.p, self._ns, self._batch = h, g, dict(p), None, batch
        self.refresh()

    def __del__(self):
        pass  # the batch frees its variants


class Batch:
    def __init__(self, geoms: Sequence[E.Geometry], params: Sequence[dict]):
        if len(geoms) != len(params) or not geoms:
            raise ValueError("one parameter set per geometry required")
        n = len(geoms)
        hs = (C.c_void_p * n)(*[g._h for g in geoms])
        rp = (A.RunParams * n)()
        for i, p in enumerate(params):
            rp[i] = A.RunParams(K=p["K"], aniso=p["aniso"], u=p["u"], tau=p["tau"], steps=int(p["steps"]),
                                avg=int(p["avg"]), every=int(p.get("every", 1) or 1),
                                storage=A.STORAGE[p.get("storage", "f32")],
                                flags=A.RUN_ALLOW_BF16 if p.get("allowBf16") else 0)
        h = C.c_void_p()
        E._check(A.load().abx_batch_create(hs, rp, n, C.byref(h)))
        self._h = h
        self.geoms = list(geoms)          # the batch borrows the geometries: keep them alive
        self.variants = [BatchVariant(self, i, g, p) for i, (g, p) in enumerate(zip(geoms, params))]

    def tune(self) -> dict:
        t = A.BatchTuning()
        E._check(A.load().abx_batch_tune(self._h, C.byref(t)))
        cands = [{"shape": t.cand_shape[i], "grid": t.cand_grid[i], "group_mb": round(t.cand_group_bytes[i] / 1e6, 1),
                  "groups": t.cand_groups[i], "ms_per_step": round(t.cand_ms[i], 4)} for i in range(t.n_candidates)]
        return {"shape": t.shape, "spw": t.spw, "min_blocks": t.min_blocks, "grid": t.grid, "ntiles": t.ntiles,
                "ms_per_step": t.ms_per_step, "group_mb": round(t.group_bytes / 1e6, 1), "groups": t.n_groups,
                "candidates": cands}

    def set_grouping(self, group_bytes: float):
        """Groups of variants of at most group_bytes of state each (0: no byte limit)."""
        E._check(A.load().abx_batch_set_grouping(self._h, float(group_bytes)))

    def set_shape(self, shape: int, grid: int):
        E._check(A.load().abx_batch_set_shape(self._h, shape, grid))

    def reset(self):
        E._check(A.load().abx_batch_reset(self._h))

    def run(self) -> np.ndarray:
        """All variants through simulate()'s schedule; returns each variant's instability step (0: stable)."""
        st = np.zeros(len(self.variants), np.int32)
        E._check(A.load().abx_batch_run(self._h, E._ptr(st)))
        return st

    @property
    def info(self) -> dict:
        i = A.BatchInfo()
        E._check(A.load().abx_batch_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in A.BatchInfo._fields_}

    def evaluate(self) -> list:
        return [v.evaluate() for v in self.variants]

    def __del__(self):
        try:
            if self._h:
                self.variants = []
                A.load().abx_batch_free(self._h)
                self._h = None
        except Exception:
            pass
