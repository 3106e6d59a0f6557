"""Build libairbox.so in-tree (airboxcalc_gb300/libairbox.so) for sm_103a.

Translation units, compiled in parallel:
  csrc/voxelize.cu   nvcc, -fmad=false (bit-exact double arithmetic of the parity voxelizer)
  csrc/lbm_exact.cu  nvcc, -fmad=false (cpuStep-exact step, float64 run, probe/evaluate/state kernels)
  csrc/lbm_fast.cu   nvcc (float32 / float16 / bfloat16 step kernels, FMA contraction allowed)
  csrc/warmstart.cu  nvcc (grid <-> network resampling, warm-start initialisation)
  csrc/nn.cu         nvcc (layer kernels of the warm-start network, forward and backward)
  csrc/nn_tc.cu      nvcc (its convolutions on the tensor cores: tcgen05, TMA, bf16 operands)
  csrc/postproc.cu   nvcc, -fmad=false (field3d, cut planes, streamlines in the reference's float64 order)
  csrc/prepare.cu    nvcc (duct, flood fill, leak, outlet, classes, kpad, segments, compact cell list)
  csrc/api.cpp       g++ -ffp-contract=off (host side of the C ABI)
  csrc/net.cpp       g++ (host side of the warm-start network: layers, training loop)
and linked with nvcc -shared (static CUDA runtime).  No torch, no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libairbox.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"] + ARCH

UNITS = [
    ("voxelize.cu", ["-fmad=false"]),
    ("lbm_exact.cu", ["-fmad=false"]),
    ("lbm_fast.cu", []),
    ("warmstart.cu", []),
    ("nn.cu", []),
    ("nn_tc.cu", []),
    ("postproc.cu", ["-fmad=false"]),
    ("prepare.cu", []),
    ("api.cpp", None),
    ("net.cpp", None),
]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libairbox.so")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _sources():
    out = [os.path.join(INCLUDE, "airbox.h"), os.path.abspath(__file__)]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False, extra_nvcc=(), out: str = None,
          build_dir: str = None) -> str:
    """Compile and link; ``extra_nvcc``/``out``/``build_dir`` build a variant elsewhere
    (e.g. with different -D tuning macros) without touching the in-tree library."""
    lib = out or LIB
    bdir = build_dir or BUILD
    if not force and out is None and up_to_date():
        return LIB
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(nvcc), "include")
    os.makedirs(bdir, exist_ok=True)

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(bdir, src + ".o")
        path = os.path.join(CSRC, src)
        if extra is None:
            cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                   "-I" + cuda_inc, "-I" + INCLUDE, "-c", path, "-o", obj]
        else:
            cmd = [nvcc] + NVCC_FLAGS + extra + list(extra_nvcc) + (["-Xptxas", "-v"] if ptxas_info else []) + \
                  ["-I" + INCLUDE, "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose or ptxas_info:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = lib + ".tmp"
    cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libairbox.so failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
