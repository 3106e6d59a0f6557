"""Benchmark of the airbox compute core on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config3|config2|config1] [--storage f32|f16] [--block B]

Default workload: config3, the largest single-GPU configuration (a
512x256x384-cell seeded airbox at dx 0.6 mm, 39.2 M fluid cells, tau 0.505,
u 0.05, 20000 LBM steps with the last 5000 averaged).

One bench step is one block of that solve's schedule: B LBM steps (default
16) of which the last round(B * avg / steps) add to the time averages (4 of
16: the 5000/20000 share), on the same continuing state.  MLUPS counts
fluid-cell updates per second, the reference's definition (src/engine.js:338).

* ``value``  - MLUPS from CUDA-event device time of the K blocks (state and
  geometry resident in HBM; the state is 4.6 GB, 36x the L2, so no flush is
  needed between blocks).
* ``e2e``    - MLUPS of whole solves through the C ABI with host buffers: each
  prepares the geometry from host triangles (H2D, GPU voxelizer, opening
  search and flood fill), runs the full schedule (all 20000 steps, progress
  probes every 500) and reads KPIs, filter map and history back.
* ``roofline`` - the fused stream+collide kernel (launches without
  averaging): 2*19*4 bytes per fluid cell per launch (float32 storage) over
  its CUDA-event launch time, against the measured HBM copy bandwidth.
* ``cpu_baseline`` - the oracle's restatement of the reference's cpuStep
  (single thread, float64 locals as in JavaScript) on the same airbox.

``--impl reference`` times the reference's CPU algorithm (no JavaScript
runtime exists on this machine, so the C restatement stands in for
src/engine.js's cpuStep) with every host core, on the same workload and the
same blocks (same ``config``).  Under torchrun the runs are independent
replicas, one per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS; time to converged γ/ζ (±1%): FP16+warm-start vs plain FP32 LBM"
RUN = dict(K=3.0, aniso=10.0, u=0.06, tau=0.51, steps=6000, avg=2000, every=150)


def workload(name: str):
    from airboxcalc_gb300 import airboxgen as ag
    if name == "config1":
        spec = ag.config1_spec()
        return spec, dict(RUN), "config1: 240x120x180 mm airbox, 70 mm inlet + 30 mm stub, dx 4 mm, 6000/2000 steps"
    if name == "config2":
        spec = ag.random_spec(1000, dx=1.5)
        return spec, dict(RUN), "config2: seeded airbox (seed 1000), dx 1.5 mm, 6000 steps / 2000 averaged"
    if name.startswith("dx2seed"):
        from airboxcalc_gb300 import warmstart as W
        spec, K = W.variant(int(name[7:]), 2.0)
        return spec, dict(W.RUN, K=K), f"seeded airbox {name[7:]} of the warm-start study, dx 2 mm, 6000/2000 steps"
    if name == "config3":
        spec = ag.grid_spec(512, 256, 384, dx=0.6)
        run = dict(RUN, tau=0.505, u=0.05, steps=20000, avg=5000, every=500)  # every: src/ui.html:502 rule
        return spec, run, "config3: 512x256x384-cell airbox, dx 0.6 mm, 20000 steps / 5000 averaged"
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples every 50 ms; only samples inside the marked timed windows count."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.windows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        t0 = time.perf_counter()
        while not self.rows and time.perf_counter() - t0 < 5.0:   # first sample in before timing starts
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append((time.perf_counter(), parts))

    def begin(self):
        self.windows.append([time.perf_counter(), None])

    def end(self):
        if self.windows and self.windows[-1][1] is None:
            self.windows[-1][1] = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        rows = [r for t, r in self.rows if any(a <= t <= (b or a) + 0.06 for a, b in self.windows)]
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks for replica runs under torchrun (gloo on the host)."""

    def __init__(self, ws: int):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel_tag: str):
    """DRAM bytes per launch of the step kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


# ------------------------------------------------------------------ CPU legs
def cpu_baseline(spec, run, nthreads: int, target_s: float = 12.0):
    """The oracle's cpuStep restatement on the workload's airbox: LBM steps from
    w_i until about target_s seconds have passed."""
    from oracle import oracle as O
    from airboxcalc_gb300 import airboxgen as ag
    og = O.prepare(ag.build_airbox(spec), spec.prepare_params(), max_cells=1e10)
    S = O.OracleSim(og, run)
    f = S.f0()
    n = 0
    t0 = time.perf_counter()
    while True:
        f = S.step(f, kind="f32", nthreads=nthreads)
        n += 1
        el = time.perf_counter() - t0
        if el >= target_s or n >= 200:
            break
    return S.NF * n / el / 1e6, n, el, S.NF


# ------------------------------------------------------------------ studies
KPI = ("gamma", "gammaCore", "lowCore", "maxToMean", "zeta")


def solve(g, run, storage, timing=True):
    """One whole simulate() + evaluate() on the GPU; returns (metrics, averages, device ms)."""
    from airboxcalc_gb300 import engine as E
    S = E.Simulation(g, {**run, "storage": storage, "allowBf16": True})
    S.set_timing(timing)
    S.run()
    res = S.evaluate()
    t = S.timing()
    return res["metrics"], S.get_acc(), t["run_ms"] + t["eval_ms"], S.NF


def study_precision(spec, run, desc, storages=("f64", "f32exact", "f32", "f16", "bf16")):
    """KPI and field error of every population storage against the float64 run
    (same airbox, same steps), with each run's MLUPS and the GB/s of its population bytes."""
    import numpy as np
    from airboxcalc_gb300 import engine as E
    g = E.prepare({"tris": __import__("airboxcalc_gb300.airboxgen", fromlist=["x"]).build_airbox(spec),
                   **spec.prepare_params(), "maxCells": 1e10})
    ref_m, ref_acc, ref_ms, NF = solve(g, run, "f64")
    ra = ref_acc.reshape(4, -1).astype(np.float64)
    rows = []
    bytes_per_update = {"f64": 304, "f32exact": 152, "f32": 152, "f16": 76, "bf16": 76}
    for st in storages:
        m, acc, ms, _ = (ref_m, ref_acc, ref_ms, NF) if st == "f64" else solve(g, run, st)
        a = acc.reshape(4, -1).astype(np.float64)
        err = {k: (m[k] - ref_m[k]) / abs(ref_m[k]) if ref_m[k] else m[k] - ref_m[k] for k in KPI}
        l2u = float(np.linalg.norm(a[:3] - ra[:3]) / np.linalg.norm(ra[:3]))
        l2r = float(np.linalg.norm(a[3] - ra[3]) / np.linalg.norm(ra[3] - 1.0))
        rows.append({"study": "precision", "workload": desc, "storage": st, "NF": NF,
                     "steps": run["steps"], "ms": round(ms, 2), "mlups": round(NF * run["steps"] / ms / 1e3, 1),
                     "population_GBs": round(bytes_per_update[st] * NF * run["steps"] / ms / 1e6, 1),
                     "kpi": {k: round(m[k], 6) for k in KPI}, "rel_err_vs_f64": {k: float(f"{v:.3e}") for k, v in err.items()},
                     "rel_l2_u_vs_f64": float(f"{l2u:.3e}"), "rel_l2_rho_minus_1_vs_f64": float(f"{l2r:.3e}")})
        print(json.dumps(rows[-1]), flush=True)
    return rows


def study_decorrelation(spec, run, desc, storages=("f32exact", "f32", "f16"),
                        checkpoints=(250, 500, 1000, 2000, 4000), window=100):
    """How the float32 / float16 fields drift from the float64 run's over a solve: all runs start from w_i on
    the same airbox; at each checkpoint every run averages the next `window` steps, and the relative L2
    difference of those averages (u, and rho - 1) to the float64 run's is reported.  A precision bias shows as
    a difference present from the first checkpoints on; the divergence of unsteady trajectories as one that
    starts at round-off level and grows with the step count."""
    import numpy as np
    from airboxcalc_gb300 import airboxgen as ag
    from airboxcalc_gb300 import engine as E
    g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
    sims = {st: E.Simulation(g, {**run, "storage": st}) for st in ("f64",) + tuple(storages)}
    done = 0
    rows = []
    for c in checkpoints:
        for S in sims.values():
            S.step(c - done)
            S.clear_acc()
            S.step(window, True)
        done = c + window
        ref = sims["f64"].get_acc().reshape(4, -1).astype(np.float64)
        row = {"study": "decorrelation", "workload": desc, "step": c, "window": window}
        for st in storages:
            a = sims[st].get_acc().reshape(4, -1).astype(np.float64)
            row[st] = {"rel_l2_u": float(f"{np.linalg.norm(a[:3] - ref[:3]) / np.linalg.norm(ref[:3]):.3e}"),
                       "rel_l2_rho_minus_1": float(f"{np.linalg.norm(a[3] - ref[3]) / np.linalg.norm(ref[3] - 1):.3e}")}
        rows.append(row)
        print(json.dumps(row), flush=True)
    return rows


def study_converge(spec, run, desc, storages=("f32", "f16", "bf16"), ladder=(600, 900, 1200, 1500, 2100, 3000, 4500, 6000)):
    """Steps and device time until gamma core and zeta are within 1 % of the plain
    float32 run on the full schedule (the reference's fixed 6000/2000 steps).
    Each ladder entry is a fresh run of S steps averaging the last S/3."""
    from airboxcalc_gb300 import airboxgen as ag
    from airboxcalc_gb300 import engine as E
    g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
    ref_m, _, ref_ms, NF = solve(g, run, "f32")
    out = []
    for st in storages:
        found = None
        for S_ in ladder:
            r = dict(run, steps=S_, avg=max(S_ // 3, 1))
            m, _, ms, _ = solve(g, r, st)
            dg = abs(m["gammaCore"] - ref_m["gammaCore"]) / abs(ref_m["gammaCore"])
            dz = abs(m["zeta"] - ref_m["zeta"]) / abs(ref_m["zeta"])
            if dg < 0.01 and dz < 0.01:
                found = (S_, ms, dg, dz)
                break
        row = {"study": "converge", "workload": desc, "storage": st, "reference_ms": round(ref_ms, 2),
               "reference_steps": run["steps"],
               "converged_steps": found[0] if found else None, "converged_ms": round(found[1], 2) if found else None,
               "err_gammaCore": float(f"{found[2]:.3e}") if found else None,
               "err_zeta": float(f"{found[3]:.3e}") if found else None,
               "speedup_vs_reference_schedule": round(ref_ms / found[1], 2) if found else None}
        out.append(row)
        print(json.dumps(row), flush=True)
    return out


# Stop rules compared by the warm-start study.  rule 0: the running average's KPIs moved less than tol over the
# last window; rule 1: batch-means standard error of the KPIs at most tol / 2 (include/airbox.h ABX_RULE_*).
WARM_RULES = (dict(settle=1000, window=500, min_avg=1000, max_steps=4000, tol=0.01, rule=0, min_windows=4),
              dict(settle=500, window=250, min_avg=1000, max_steps=6000, tol=0.01, rule=1, min_windows=4),
              dict(settle=1000, window=500, min_avg=2000, max_steps=6000, tol=0.01, rule=1, min_windows=4))
# Adaptive runs without the restart: the stop rule, and where it has not fired by max_steps the running average is
# reported as it is (no fallback to the full schedule from f = w_i).
ADAPTIVE_RULES = (dict(settle=500, window=250, min_avg=1000, max_steps=2500, tol=0.01, rule=1, min_windows=4, fallback=False),
                  dict(settle=500, window=250, min_avg=1000, max_steps=3000, tol=0.01, rule=1, min_windows=4, fallback=False),
                  dict(settle=750, window=250, min_avg=1000, max_steps=3000, tol=0.01, rule=0, min_windows=4, fallback=False))
# Fixed step budgets (no stop test: a tolerance no window misses, two windows): settle S steps, then average A;
# S + A = 1250, 1500, 2000 and 3000 steps, i.e. 4.8x, 4x, 3x and 2x fewer than the reference's 6000.
BUDGET_RULES = tuple(dict(settle=s, window=a // 2, min_avg=a, max_steps=s + a, tol=1e9, rule=0, min_windows=2)
                     for s, a in ((250, 1000), (500, 1000), (500, 1500), (1000, 2000)))


def _rel_err(m, ref):
    return (abs(m["gammaCore"] - ref["gammaCore"]) / abs(ref["gammaCore"]),
            abs(m["zeta"] - ref["zeta"]) / abs(ref["zeta"]))


def _feq_host(acc, NF):
    """Equilibrium populations f[q*NF + a] (float32) of the averaged fields acc[c*NF + a] (cpuStep's feq)."""
    import numpy as np
    cx = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
    cy = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
    cz = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    a = acc.reshape(4, NF).astype(np.float64)
    ux, uy, uz, rho = a
    u2 = ux * ux + uy * uy + uz * uz
    f = np.empty((19, NF))
    for q in range(19):
        cu = cx[q] * ux + cy[q] * uy + cz[q] * uz
        f[q] = w[q] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u2)
    return f.astype(np.float32).ravel()


def study_warmstart(seeds, weights: str, rules=WARM_RULES, uniform: bool = True, noise: bool = True,
                    perfect: bool = True, quiet: bool = False):
    """Time to converged gamma core / zeta: float16 storage + learned warm start + convergence run
    (abx_sim_solve_warm) against the plain float32 run on the reference's fixed schedule, on held-out
    seeded airboxes at dx 2 mm.  Wall times are host clocks around the solve (prepare excluded), each
    taken after one untimed solve of the same arm on the same simulation object (CUDA graphs built).
    With `uniform`, the same convergence run from f = w_i (float16) shows what the network adds.  With
    `noise`, the plain float32 run continued to 8000 steps (averaging 6000-8000) measures how far the
    reference's own KPIs move between consecutive 2000-step windows: the noise floor of the +-1 % test.  With
    `perfect`, the convergence run starts from the equilibrium of the plain run's own time-averaged field (what an
    exact network would predict; the upload is not timed): the ceiling of the learned warm start."""
    from airboxcalc_gb300 import airboxgen as ag
    from airboxcalc_gb300 import engine as E
    from airboxcalc_gb300 import warmstart as W
    net = W.Net.load(weights)
    rows = []
    for seed in seeds:
        spec, K = W.variant(seed, 2.0)
        run = dict(W.RUN, K=K)
        try:
            g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
            P = E.Simulation(g, run)
            P.run()
            P.reset()
            t0 = time.perf_counter()
            P.run()
            ref = P.evaluate()["metrics"]
            plain_ms = (time.perf_counter() - t0) * 1e3
        except E.AirboxError as e:
            rows.append({"seed": seed, "skipped": e.code})
            continue
        row = {"seed": seed, "K": K, "NF": P.NF, "plain_f32_ms": round(plain_ms, 2),
               "ref": {"gammaCore": ref["gammaCore"], "zeta": ref["zeta"]}}
        f_perfect = _feq_host(P.get_acc(), P.NF) if perfect else None
        if noise:
            # the plain run's next 2000-step window (noise floor of the +-1 % test against the 6000/2000 KPIs), then
            # the same run averaged over 8000 steps (6000-14000): the long-window reference
            P.clear_acc()
            P.step(2000, True)
            eg, ez = _rel_err(P.evaluate()["metrics"], ref)
            row["noise_f32"] = {"ms": plain_ms, "steps": 8000, "err_gammaCore": float(f"{eg:.3e}"),
                                "err_zeta": float(f"{ez:.3e}")}
            P.step(6000, True)
            long_ref = P.evaluate()["metrics"]
            row["ref_long"] = {"gammaCore": long_ref["gammaCore"], "zeta": long_ref["zeta"]}
            eg, ez = _rel_err(ref, long_ref)
            row["plain_vs_long"] = {"ms": plain_ms, "steps": 6000, "err_gammaCore": float(f"{eg:.3e}"),
                                    "err_zeta": float(f"{ez:.3e}")}
        del P
        S = E.Simulation(g, dict(run, storage="f16"))
        for i, rule in enumerate(rules):
            if rule.get("fallback", True):
                rule = {k: v for k, v in rule.items() if k != "fallback"}
                W.solve_warm(S, net, **rule)
                r = W.solve_warm(S, net, **rule)
                eg, ez = _rel_err(r["metrics"], ref)
                row[f"warm{i}"] = {"ms": round(r["total_ms"], 2), "steps": r["steps"], "fell_back": r["fell_back"],
                                   "infer_ms": round(r["infer_ms"], 3), "err_gammaCore": float(f"{eg:.3e}"),
                                   "err_zeta": float(f"{ez:.3e}")}
            else:
                # warm start and convergence run, the running average reported even where the rule did not fire
                rule = {k: v for k, v in rule.items() if k != "fallback"}
                try:
                    for timed in (False, True):
                        S.reset()
                        t0 = time.perf_counter()
                        W.warm_start(S, net)
                        r = W.converge(S, **rule)
                        ms = (time.perf_counter() - t0) * 1e3
                    fell = 0
                except E.AirboxError:
                    # the warm-started run went unstable: the reference's start and schedule, as solve_warm does
                    # (the time counts the attempt that failed)
                    t_fail = (time.perf_counter() - t0) * 1e3
                    S.reset()
                    t1 = time.perf_counter()
                    S.run()
                    r = {"metrics": S.evaluate()["metrics"], "steps": run["steps"], "converged": False}
                    ms, fell = t_fail + (time.perf_counter() - t1) * 1e3, 1
                eg, ez = _rel_err(r["metrics"], ref)
                row[f"warm{i}"] = {"ms": round(ms, 2), "steps": r["steps"], "fell_back": fell, "converged": r["converged"],
                                   "err_gammaCore": float(f"{eg:.3e}"), "err_zeta": float(f"{ez:.3e}")}
            if "ref_long" in row:
                lg, lz = _rel_err(r["metrics"], row["ref_long"])
                row[f"warm{i}"].update(err_long_gammaCore=float(f"{lg:.3e}"), err_long_zeta=float(f"{lz:.3e}"))
        if perfect:
            for i, rule in enumerate(rules):
                rule = {k: v for k, v in rule.items() if k != "fallback"}
                S.reset()
                S.set_f(f_perfect)
                W.converge(S, **rule)
                S.reset()
                S.set_f(f_perfect)
                t0 = time.perf_counter()
                r = W.converge(S, **rule)
                ms = (time.perf_counter() - t0) * 1e3
                eg, ez = _rel_err(r["metrics"], ref)
                row[f"perfect{i}"] = {"ms": round(ms, 2), "steps": r["steps"], "converged": r["converged"],
                                      "err_gammaCore": float(f"{eg:.3e}"), "err_zeta": float(f"{ez:.3e}")}
        if uniform:
            rule = {k: v for k, v in rules[0].items() if k != "fallback"}
            S.reset()
            W.converge(S, **rule)
            S.reset()
            t0 = time.perf_counter()
            r = W.converge(S, **rule)
            ms = (time.perf_counter() - t0) * 1e3
            eg, ez = _rel_err(r["metrics"], ref)
            row["uniform0"] = {"ms": round(ms, 2), "steps": r["steps"], "converged": r["converged"],
                               "err_gammaCore": float(f"{eg:.3e}"), "err_zeta": float(f"{ez:.3e}")}
        rows.append(row)
        if not quiet:
            print(json.dumps(row), flush=True)
    done = [r for r in rows if "skipped" not in r]

    def summary(key):
        xs = [r[key] for r in done if key in r]
        if not xs:
            return None
        ok = [max(x["err_gammaCore"], x["err_zeta"]) < 0.01 for x in xs]
        sp = [r["plain_f32_ms"] / r[key]["ms"] for r in done if key in r]
        out = {"n": len(xs), "within_1pct": round(sum(ok) / len(xs), 3),
               "within_1pct_of_long_reference": (round(sum(max(x["err_long_gammaCore"], x["err_long_zeta"]) < 0.01
                                                           for x in xs) / len(xs), 3)
                                                 if "err_long_zeta" in xs[0] else None),
               "median_speedup_vs_plain_f32": round(statistics.median(sp), 2),
               "mean_wall_speedup": round(sum(r["plain_f32_ms"] for r in done) / sum(x["ms"] for x in xs), 2),
               "median_err_gammaCore": float(f"{statistics.median(x['err_gammaCore'] for x in xs):.3e}"),
               "median_err_zeta": float(f"{statistics.median(x['err_zeta'] for x in xs):.3e}"),
               "median_steps": statistics.median(x["steps"] for x in xs)}
        if "fell_back" in xs[0]:
            out["fallback_rate"] = round(sum(x["fell_back"] for x in xs) / len(xs), 3)
        return out

    summ = {"study": "warmstart", "seeds": f"{min(seeds)}..{max(seeds)}", "evaluated": len(done),
            "skipped_unstable_or_leaking": len(rows) - len(done), "weights": os.path.relpath(weights, ROOT),
            "rules": [dict(r) for r in rules]}
    for i in range(len(rules)):
        summ[f"warm{i}_f16"] = summary(f"warm{i}")
    if perfect:
        for i in range(len(rules)):
            summ[f"perfect{i}_f16"] = summary(f"perfect{i}")
    if uniform:
        summ["uniform0_f16"] = summary("uniform0")
    if noise:
        summ["noise_floor_f32_next_window"] = summary("noise_f32")
        summ["plain_6000_2000_vs_long_reference"] = summary("plain_vs_long")
    print(json.dumps(summ), flush=True)
    return summ, rows


def batch_variants(n: int, seed0: int = 7000, dx_lo: float = 2.0, dx_hi: float = 4.0):
    """The variant table of the batched run: seeded airboxes with dx in [dx_lo, dx_hi) mm (default [2, 4)) and K in
    {1.5, 3, 6}."""
    from airboxcalc_gb300 import airboxgen as ag
    out = []
    for v in range(n):
        seed = seed0 + v
        dx = round(dx_lo + (dx_hi - dx_lo) * ((seed * 0.6180339887498949) % 1.0), 3)
        out.append((seed, ag.random_spec(seed, dx=dx), (1.5, 3.0, 6.0)[seed % 3], dx))
    return out


def net_flops(res: int, base: int, levels: int, batch: int) -> float:
    """Multiply-add FLOPs (2 per MAC) of one training step of the warm-start network: every convolution's
    forward, data gradient (all but the first layer's) and weight gradient."""
    chans = [base << l for l in range(levels)]
    conv, d, c = [], res, 9
    for l in range(levels):
        d = d if l == 0 else d // 2
        conv += [(c, chans[l], d), (chans[l], chans[l], d)]
        c = chans[l]
    for l in range(levels - 2, -1, -1):
        d *= 2
        conv += [(chans[l + 1], chans[l], d), (chans[l], chans[l], d)]
    conv.append((chans[0], 4, d))
    total = 0.0
    for i, (cin, cout, do) in enumerate(conv):
        f = 2.0 * 27 * cin * cout * do ** 3 * batch
        total += f * (2 if i == 0 else 3)
    return total


def study_net(batch: int = 8, iters: int = 10, modes=("f32", "tc"), res: int = 64, base: int = 16, levels: int = 4):
    """One training step (forward, loss, backward) of the warm-start network at its shipped shape on synthetic
    inputs, timed per convolution path: the float32 kernels and the tensor cores (bf16 operands, float32
    accumulation).  Reports ms per step and TFLOP/s of the convolutions' multiply-adds."""
    import torch
    from airboxcalc_gb300 import warmstart as W
    rng = np.random.default_rng(0)
    flops = net_flops(res, base, levels, batch)
    out = {"study": "net", "res": res, "base": base, "levels": levels, "batch": batch, "iters": iters,
           "tflop_per_step": round(flops / 1e12, 4)}
    for mode in modes:
        net = W.Net(res, base, levels, seed=3)
        net.set_tensor_cores(mode == "tc")
        x = torch.from_numpy(rng.standard_normal((batch, net.n_in, res, res, res)).astype(np.float32)).cuda()
        t = torch.from_numpy(rng.standard_normal((batch, 4, res, res, res)).astype(np.float32)).cuda()
        m = torch.ones((batch, res, res, res), dtype=torch.float32, device="cuda")
        pred = torch.empty((batch, 4, res, res, res), dtype=torch.float32, device="cuda")
        grad = torch.empty(net.n_params, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()

        def step():
            return net.forward_backward(x.data_ptr(), t.data_ptr(), m.data_ptr(), batch, 1.0 / m.numel(),
                                        pred.data_ptr(), grad.data_ptr())

        step()
        t0 = time.perf_counter()
        for _ in range(iters):
            step()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / iters * 1e3
        out[mode] = {"ms_per_step": round(ms, 3), "tflops": round(flops / ms / 1e9, 1)}
        del net
    if "f32" in out and "tc" in out:
        out["speedup"] = round(out["f32"]["ms_per_step"] / out["tc"]["ms_per_step"], 2)
    print(json.dumps(out), flush=True)
    return out


def study_batch(n: int = 64, storage: str = "f16", quiet: bool = False, dx_range=(2.0, 4.0)):
    """Batched variants: every seeded airbox alone in float32 (the reference's method, one solve at a
    time), alone in `storage`, and all together in one batched run (tuned shape, one launch per step).
    Reports aggregate MLUPS of each and each variant's KPI error against its float32 run."""
    from airboxcalc_gb300 import airboxgen as ag
    from airboxcalc_gb300 import batch as BT
    from airboxcalc_gb300 import engine as E
    geoms, params, rows, skipped = [], [], [], []
    t32 = t16 = 0.0
    cells = 0
    for seed, spec, K, dx in batch_variants(n, dx_lo=dx_range[0], dx_hi=dx_range[1]):
        run = dict(RUN, K=K)
        try:
            g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
            S = E.Simulation(g, run)
            S.set_timing(True)
            S.run()
            ref = S.evaluate()["metrics"]
        except E.AirboxError as e:
            skipped.append({"seed": seed, "dx": dx, "code": e.code})
            continue
        t = S.timing()
        t32 += t["run_ms"]
        S16 = E.Simulation(g, dict(run, storage=storage, allowBf16=True))
        S16.set_timing(True)
        S16.run()
        t16 += S16.timing()["run_ms"]
        del S, S16
        geoms.append(g)
        params.append(dict(run, storage=storage, allowBf16=True))
        rows.append({"seed": seed, "dx": dx, "K": K, "NF": g.nf, "ref": ref})
        cells += g.nf
    B = BT.Batch(geoms, params)
    tuning = B.tune()
    B.run()
    B.reset()
    st = B.run()
    info = B.info
    errs = []
    for r, v, s_ in zip(rows, B.variants, st):
        m = v.evaluate()["metrics"]
        eg, ez = _rel_err(m, r["ref"])
        errs.append(max(eg, ez))
        r.update({"err_gammaCore": float(f"{eg:.3e}"), "err_zeta": float(f"{ez:.3e}"), "unstable_step": int(s_)})
        del r["ref"]
        if not quiet:
            print(json.dumps(r), flush=True)
    upd = cells * RUN["steps"]
    out = {"study": "batch", "dx_mm": list(dx_range), "variants": len(rows), "skipped_unstable_or_leaking": len(skipped),
           "cells_min": min(r["NF"] for r in rows), "cells_max": max(r["NF"] for r in rows), "cells_total": cells,
           "storage": storage, "steps": RUN["steps"], "avg": RUN["avg"],
           "batched_mlups": round(upd / (info["run_ms"] * 1e-3) / 1e6, 1),
           "one_at_a_time_mlups": {storage: round(upd / (t16 * 1e-3) / 1e6, 1), "f32": round(upd / (t32 * 1e-3) / 1e6, 1)},
           "batched_run_ms": round(info["run_ms"], 1), "kernel_launches": info["kernel_launches"],
           "tuning": {k: tuning[k] for k in ("shape", "spw", "min_blocks", "grid", "ntiles", "ms_per_step", "group_mb",
                                             "groups")},
           "tuning_candidates": tuning["candidates"],
           "kpi_err_vs_individual_f32": {"max": float(f"{max(errs):.3e}"),
                                         "median": float(f"{statistics.median(errs):.3e}"),
                                         "within_0.5pct": round(sum(e < 0.005 for e in errs) / len(errs), 3),
                                         "within_1pct": round(sum(e < 0.01 for e in errs) / len(errs), 3)}}
    print(json.dumps(out), flush=True)
    return out


def block_shape(run, block: int):
    """(plain, averaged) LBM steps of one bench step: the schedule's averaged share of `block` steps."""
    nacc = max(1, round(block * run["avg"] / run["steps"])) if run["avg"] > 0 else 0
    return block - nacc, nacc


def bench_config(desc, grid, NF, run, block, storage, ws):
    """The `config` object of the bench line; both arms print the same one."""
    plain, nacc = block_shape(run, block)
    state_bytes = (19 + 4) * 4 * NF   # float32 populations (one A-A array) and averages of the fluid cells
    return {"workload": desc, "grid": list(grid), "NF": int(NF), "schedule": {"steps": run["steps"],
            "avg": run["avg"], "every": run["every"], "tau": run["tau"], "u": run["u"]},
            "lbm_steps_per_bench_step": block, "averaged_steps_per_bench_step": nacc, "storage": storage,
            "state_bytes": int(state_bytes),
            "l2": "state larger than the 129 MB L2, no flush needed" if state_bytes > 129e6 else "state smaller than L2",
            "e2e": "whole solves (prepare from host triangles, full schedule, evaluate and read-back)",
            "parallelism": f"replicas x{ws}"}


def reference_arm(a, spec, run, desc, rank):
    """--impl reference: the C restatement of cpuStep (src/engine.js:266-321) on every host core, on the same
    airbox and the same blocks of the schedule as our arm."""
    if rank != 0:
        return 0
    from oracle import oracle as O
    from airboxcalc_gb300 import airboxgen as ag
    O.build()
    cores = os.cpu_count() or 1
    og = O.prepare(ag.build_airbox(spec), spec.prepare_params(), max_cells=1e10)
    S = O.OracleSim(og, run)
    plain, nacc = block_shape(run, a.block)
    f = S.f0()
    acc = np.zeros(4 * S.NF, np.float32)

    def block():
        nonlocal f
        for _ in range(plain):
            f = S.step(f, kind="f32", nthreads=cores)
        for _ in range(nacc):
            f = S.step(f, acc=acc, kind="f32", nthreads=cores)

    for _ in range(a.warmup):
        block()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        block()
    el = time.perf_counter() - t0
    v = S.NF * a.block * a.steps / el / 1e6
    sample = (f"{a.block} LBM steps per bench step ({plain} plain, {nacc} adding to the averages) of the workload "
              f"airbox (NF={S.NF}) on a continuing state from w_i")
    line = {"metric": METRIC, "value": round(v, 3), "unit": "MLUPS", "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(el / a.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64-locals/f32-storage", "data": "synthetic",
            "config": bench_config(desc, (og.nx, og.ny, og.nz), S.NF, run, a.block, "f32", a.gpus),
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 3), "unit": "MLUPS", "cores": cores, "kind": "port",
                             "sample": sample + "; C restatement of src/engine.js cpuStep (no JavaScript "
                             "runtime here or on the GPU host), OpenMP over cells"},
            "e2e": {"value": round(v, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config3",
                    help="config3 (default), config2, config1, or dx2seedN (airbox N of the warm-start study)")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16"])
    ap.add_argument("--block", type=int, default=16, help="LBM steps per bench step")
    ap.add_argument("--e2e-solves", type=int, default=2, help="whole end-to-end solves timed for e2e")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-warm-start", action="store_true", help="skip the warm-start sample of the bench line")
    ap.add_argument("--study", choices=["precision", "converge", "warmstart", "batch", "decorrelation", "net"],
                    default=None,
                    help="instead of the bench line: KPI error per storage vs float64, steps/time to converged "
                         "KPIs, the learned warm start on held-out airboxes, the batched variant table, the "
                         "growth of the float32/float16 vs float64 field difference over a solve, or one "
                         "training step of the warm-start network on the float32 kernels and the tensor cores")
    ap.add_argument("--batch-dx", default="2:4", help="--study batch: cell size range lo:hi (mm) of the variant table")
    ap.add_argument("--net-batch", type=int, default=8, help="batch of --study net")
    ap.add_argument("--net-iters", type=int, default=10, help="timed training steps of --study net")
    ap.add_argument("--net-modes", default="f32,tc", help="convolution paths of --study net")
    ap.add_argument("--seeds", default="6000:6200", help="held-out seed range a:b of --study warmstart")
    ap.add_argument("--warm-rules", default="stop", choices=["stop", "budget", "adaptive"],
                    help="--study warmstart: the stop rules with the restart fallback, fixed step budgets (settle + "
                         "average) without a stop test, which map the accuracy of the learned and of a perfect start "
                         "against the budget, or the stop rules without the restart")
    ap.add_argument("--storages", default="f64,f32exact,f32,f16,bf16", help="storages of --study precision")
    ap.add_argument("--weights", default=None, help="warm-start network weights (.npz)")
    a = ap.parse_args()
    ws, rank, local = dist_env()
    spec, run, desc = workload(a.workload)
    if a.study == "precision":
        study_precision(spec, run, desc, tuple(a.storages.split(",")))
        return 0
    if a.study == "converge":
        study_converge(spec, run, desc)
        return 0
    if a.study == "decorrelation":
        study_decorrelation(spec, run, desc)
        return 0
    if a.study == "batch":
        study_batch(64, "f16", dx_range=tuple(float(v) for v in a.batch_dx.split(":")))
        return 0
    if a.study == "net":
        study_net(a.net_batch, a.net_iters, tuple(a.net_modes.split(",")))
        return 0
    if a.study == "warmstart":
        from airboxcalc_gb300 import warmstart as W
        lo, hi = map(int, a.seeds.split(":"))
        if a.warm_rules == "budget":
            study_warmstart(range(lo, hi), a.weights or W.WEIGHTS, rules=BUDGET_RULES, uniform=False, noise=False)
        elif a.warm_rules == "adaptive":
            study_warmstart(range(lo, hi), a.weights or W.WEIGHTS, rules=ADAPTIVE_RULES, uniform=False, noise=False,
                            perfect=False)
        else:
            study_warmstart(range(lo, hi), a.weights or W.WEIGHTS)
        return 0
    if a.impl == "reference":
        return reference_arm(a, spec, run, desc, rank)
    return ours_arm(a, spec, run, desc, ws, rank, local)


def ours_arm(a, spec, run, desc, ws, rank, local):
    from airboxcalc_gb300 import airboxgen as ag
    from airboxcalc_gb300 import engine as E
    dist = Dist(ws)
    device = local if ws > 1 else 0
    tris = ag.build_airbox(spec)
    p = {**spec.prepare_params(), "maxCells": 1e10, "device": device}
    runp = {**run, "storage": a.storage}
    g = E.prepare({"tris": tris, **p})
    S = E.Simulation(g, runp)
    NF = S.NF
    S.set_timing(True)
    plain, nacc = block_shape(run, a.block)

    def block():
        S.step(plain)
        if nacc:
            S.step(nacc, accumulate=True)

    for _ in range(a.warmup):
        block()
    sampler = ClockSampler(device)
    sampler.start()
    dist.barrier()
    t_before = S.timing()
    sampler.begin()
    t_wall0 = time.perf_counter()
    for _ in range(a.steps):
        block()
    wall = time.perf_counter() - t_wall0
    sampler.end()
    dist.barrier()
    t_after = S.timing()
    S.refresh()
    d = {k: t_after[k] - t_before[k] for k in t_after}
    t_dev_max = dist.max(d["step_ms"])
    units = dist.sum(NF * a.block * a.steps)
    value = units / (t_dev_max * 1e-3) / 1e6
    ms_per_step = t_dev_max / a.steps

    # end to end through the C ABI with host buffers: whole solves from host triangles
    e2e_times, h2d, d2h, e2e_kernels, kpis = [], 0, 0, 0, None
    for i in range(a.e2e_solves):
        sampler.begin()
        t0 = time.perf_counter()
        g2 = E.prepare({"tris": tris, **p})
        S2 = E.Simulation(g2, runp)
        S2.run()
        r2 = S2.evaluate()
        el = time.perf_counter() - t0
        sampler.end()
        e2e_times.append(el)
        gi, t2 = g2.info, S2.timing()
        h2d = gi.h2d_bytes + t2["h2d_bytes"]
        d2h = gi.d2h_bytes + t2["d2h_bytes"]
        e2e_kernels = gi.kernel_launches + t2["kernel_launches"]
        kpis = r2["metrics"]
        del S2, g2
    clocks = sampler.stop()
    e2e_t = dist.max(sum(e2e_times)) / max(len(e2e_times), 1)
    e2e = dist.sum(NF * run["steps"]) / e2e_t / 1e6 if e2e_times else 0.0

    # roofline of the fused step kernel (launches without averaging)
    bytes_per_cell = 2 * 19 * (4 if a.storage == "f32" else 2)
    avg_launch_ms = d["step_ms_plain"] / max(d["step_launches_plain"], 1)
    achieved = bytes_per_cell * NF / (avg_launch_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = ncu_traffic(f"lbm_step_{a.storage}_{a.workload}")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "kernel": (f"aa_vec_kernel<{a.storage}, {S.info.vec_width} cells per thread> (fused pull-stream+collide, "
                           f"A-A in place, {S.info.vec_interior_cells} of {NF} fluid cells in vector blocks)"
                           if S.info.vec_width else
                           f"aa_step_kernel<{a.storage}> (fused pull-stream+collide, A-A in place)"),
                "bytes_per_launch": bytes_per_cell * NF, "avg_launch_us": round(avg_launch_ms * 1e3, 3),
                "launches_timed": int(d["step_launches_plain"])}

    line = {"metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": a.storage, "data": "synthetic",
            "config": bench_config(desc, (g.nx, g.ny, g.nz), NF, run, a.block, a.storage, ws),
            "device_state_bytes": int(S.info.state_bytes),
            "kpis_e2e_solve": ({k: round(kpis[k], 6) for k in ("gamma", "gammaCore", "lowCore", "maxToMean", "zeta")}
                               if kpis else None),
            "e2e": {"value": round(e2e, 1), "unit": "MLUPS", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_t * 1e3, 3),
                    "step": f"one whole solve ({run['steps']} LBM steps), {a.e2e_solves} timed"},
            "roofline": roofline,
            "gpu_launches": int(d["kernel_launches"]),
            "gpu_launches_e2e_per_step": int(e2e_kernels),
            "wall_s_timed": round(wall + sum(e2e_times), 3),
            "clocks": clocks}
    if rank == 0 and not a.no_cpu_baseline:
        v, n, el, nf = cpu_baseline(spec, run, 1)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "MLUPS", "cores": 1, "kind": "port",
                                "sample": f"{n} LBM steps of the same airbox (NF={nf}) from w_i in {el:.1f} s, "
                                          "oracle restatement of src/engine.js cpuStep (float64 locals), 1 thread"}
    if rank == 0 and not a.no_warm_start:
        from airboxcalc_gb300 import warmstart as W
        if os.path.exists(W.WEIGHTS):
            summ, _ = study_warmstart(range(6000, 6048), W.WEIGHTS, rules=WARM_RULES[:1], uniform=False,
                                      noise=False, perfect=False, quiet=True)
            w = summ["warm0_f16"]
            line["warm_start"] = {
                "what": "time to converged gamma core / zeta: float16 + learned warm start + convergence run vs the "
                        "plain float32 run (6000/2000 steps), host wall time per solve, held-out seeded airboxes "
                        "6000-6047 at dx 2 mm (the full 200-seed study: bench.py --study warmstart)",
                "airboxes": w["n"], "median_speedup_vs_plain_f32": w["median_speedup_vs_plain_f32"],
                "within_1pct_both_kpis": w["within_1pct"], "median_err_gammaCore": w["median_err_gammaCore"],
                "median_err_zeta": w["median_err_zeta"], "fallback_rate": w["fallback_rate"],
                "median_steps": w["median_steps"], "rule": WARM_RULES[0]}
    if rank == 0:
        print(json.dumps(line))
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
