"""Generate the golden fixtures in tests/golden/ by running the reference's own
Python CLI, airbox_cfd.py (Awsmqt/AirboxCalc), imported from the reference
checkout given by --reference or by the AIRBOXCALC_REFERENCE environment variable
(one of the two is required).

The reference ships no tests, fixtures or STL files.  What its Python code can
pin for the compute core:

* ``load_stl`` (airbox_cfd.py:60-68) - binary and ASCII STL parsing;
* ``to_local`` (airbox_cfd.py:70-80) - the axis permutation of makeFrame for
  zero yaw;
* ``voxelize`` (airbox_cfd.py:83-114) - the same parity fill along local Z
  with the same jitter as src/engine.js:45-93;
* ``main`` (airbox_cfd.py:143-223) run for one step - the 27->1 downsample
  (mean >= 0.25, i.e. at least 7 of 27), the inlet duct, the closed bottom and
  the 6-connected flood from the inlet, saved as the solid and fluid masks;
* ``report`` (airbox_cfd.py:296-314) - gamma, gamma core, the core shares under
  50 % / over 150 %, reverse flow, peak-to-mean and zeta, computed by the CLI on
  its own averaged fields of a 60-step run (fields and KPIs both stored, for
  two geometries), which pins the formulas of evaluate() (src/engine.js:632-660).

The JS path stores voxel hits as float32 and tests ``ceil(z/h - 0.5)``, the
Python path keeps float64 and tests ``zc >= z``; the two agree unless a face
plane lies within float32 rounding of a fine-cell centre, so the fixture
geometries use dimensions that are not multiples of the cell size.  main()
imports matplotlib only in report(); a stand-in module is installed for that
call (matplotlib is not installed here).

Run:  python tests/golden/make_golden.py --reference PATH
      (or AIRBOXCALC_REFERENCE=PATH python tests/golden/make_golden.py)
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import math
import os
import sys
import tempfile
import types
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from airboxcalc_gb300 import airboxgen as ag  # noqa: E402

# Geometries with dimensions that are not multiples of the cell size (no ties).
CASES = {
    "small_baffle": dict(spec=dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0,
                                   dx=5.0, baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})),
    "wide_low": dict(spec=dict(Lx=201.13, Ly=88.71, Lz=151.37, t=3.07, d_in=55.21, stub=30.41, pleat=40.0,
                               dx=4.0, hole_x=88.33)),
    "fine_cells": dict(spec=dict(Lx=96.17, Ly=71.43, Lz=80.29, t=2.93, d_in=30.11, stub=15.37, pleat=30.0,
                                 dx=2.5, baffle={"z": 33.71, "x0": 40.13, "x1": 93.24, "y0": 55.07})),
}


# geometries whose report() KPIs are stored (on the CLI's own averaged fields of a 60-step run)
REPORT_CASES = ("small_baffle", "wide_low")

# report() result keys (airbox_cfd.py:360-363) in the order stored in the fixture
REPORT_KPIS = ("gamma", "gamma_ohne_randzellen", "anteil_unter_50pct_kern", "anteil_ueber_150pct_kern",
               "anteil_rueckstroemung", "max_zu_mittel", "zeta_rohluftseite")


def _fake_matplotlib():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = mock.MagicMock()
    plt.subplots.return_value = (mock.MagicMock(), mock.MagicMock())
    colors = mock.MagicMock()
    return {"matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.colors": colors}


def run_main(R, stl_path, spec: ag.AirboxSpec, workdir, steps=1, avg=1):
    """main() of the CLI; returns its saved fields and its report() KPIs (unrounded: the module's `round`
    is replaced by the identity for the call)."""
    argv = ["airbox_cfd.py", stl_path, "--dx", str(spec.dx), "--steps", str(steps), "--avg", str(avg),
            "--pleat", str(spec.pleat), "--tag", "g"]
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        with mock.patch.object(sys, "argv", argv), mock.patch.dict(sys.modules, _fake_matplotlib()), \
                mock.patch.object(R, "round", lambda x, n=None: x, create=True), \
                contextlib.redirect_stdout(io.StringIO()):
            R.main()
        d = np.load(os.path.join(workdir, "airbox_result_g.npz"))
        out = {k: d[k] for k in ("solid", "fluid", "ux", "uy", "uz", "rho")}
        out["report"] = json.load(open(os.path.join(workdir, "airbox_ergebnis_g.json")))
        return out
    finally:
        os.chdir(cwd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("AIRBOXCALC_REFERENCE"),
                    help="checkout of the reference holding airbox_cfd.py (default: $AIRBOXCALC_REFERENCE)")
    a = ap.parse_args()
    if not a.reference:
        ap.error("give the reference checkout with --reference PATH or AIRBOXCALC_REFERENCE")
    sys.dont_write_bytecode = True   # leave the reference checkout untouched
    sys.path.insert(0, a.reference)
    import airbox_cfd as R  # the reference's own module

    out = {}
    # ---- STL parsing: a coarse airbox as binary and as ASCII
    spec = ag.AirboxSpec(**{**CASES["small_baffle"]["spec"], "segments": 12})
    tris = ag.build_airbox(spec)
    with tempfile.TemporaryDirectory() as td:
        fb, fa = os.path.join(td, "b.stl"), os.path.join(td, "a.stl")
        open(fb, "wb").write(ag.to_binary_stl(tris))
        open(fa, "wb").write(ag.to_ascii_stl(tris))
        out["stl_binary"] = np.frombuffer(open(fb, "rb").read(), np.uint8)
        out["stl_ascii"] = np.frombuffer(open(fa, "rb").read(), np.uint8)
        out["stl_binary_parsed"] = R.load_stl(fb).astype(np.float32).reshape(-1)
        out["stl_ascii_parsed"] = R.load_stl(fa).astype(np.float32).reshape(-1)
    # ---- frame: every axis/sign combination on seeded points
    rng = np.random.default_rng(5)
    pts = rng.uniform(-200, 200, size=(64, 3, 3)).astype(np.float32).astype(float)
    combos = []
    for dax in "xyz":
        for dsg in "+-":
            for face in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax"):
                if face[0] == dax:
                    continue
                seal = float(rng.uniform(-20, 20))
                loc = R.to_local(pts, dax, dsg, face, seal).reshape(-1, 3)
                combos.append((dax, dsg, face, seal))
                out[f"frame_{dax}{'p' if dsg == '+' else 'm'}_{face}"] = np.concatenate(
                    [np.array([seal]), loc.ravel()])
    out["frame_points"] = pts.reshape(-1, 3)
    # ---- voxelizer and masks
    with tempfile.TemporaryDirectory() as td:
        for name, case in CASES.items():
            spec = ag.AirboxSpec(**case["spec"])
            ag.check_spec(spec)
            tris = ag.build_airbox(spec)
            stl = os.path.join(td, name + ".stl")
            open(stl, "wb").write(ag.to_binary_stl(tris))
            T = R.to_local(R.load_stl(stl), "y", "+", "zmin", 0.0)
            P = T.reshape(-1, 3)
            mn, mx = P.min(0), P.max(0)
            h = spec.dx
            origin = np.array([mn[0] - h, mn[1] - h, mn[2] - 10 * h])
            shape = tuple(int(math.ceil((mx[i] - origin[i] + h) / h)) for i in range(3))
            fine = R.voxelize(T, origin, tuple(s * 3 for s in shape), h / 3)
            masks = run_main(R, stl, spec, td)
            if name in REPORT_CASES:
                # report()'s KPIs (airbox_cfd.py:301-314) on the CLI's own averaged fields of a 60-step run
                run = run_main(R, stl, spec, td, steps=60, avg=20)
                for k in ("ux", "uy", "uz", "rho"):
                    out[f"report_{name}_{k}"] = run[k].astype(np.float32)
                rep = run["report"]
                out[f"report_{name}_kpi"] = np.array([rep[k] for k in REPORT_KPIS], np.float64)
            out[f"vox_{name}_shape"] = np.array(fine.shape, np.int64)
            out[f"vox_{name}_fine"] = np.packbits(fine.ravel())
            out[f"vox_{name}_solid"] = np.packbits(masks["solid"].ravel())
            out[f"vox_{name}_fluid"] = np.packbits(masks["fluid"].ravel())
            out[f"vox_{name}_coarse_shape"] = np.array(masks["fluid"].shape, np.int64)
    path = os.path.join(HERE, "airbox_cfd_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
