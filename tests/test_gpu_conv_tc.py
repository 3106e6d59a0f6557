"""The tensor-core convolutions layer by layer: tests/native/conv_tc_check.cu
(compiled here with nvcc for sm_103a) runs every convolution shape of the
warm-start network through nn_tc.cu and through the float32 kernels of nn.cu
with bfloat16-representable operands, where the two must agree to float32
summation error (relative L2 < 1e-5) in the output, the data gradient, the
weight gradient and the bias gradient; then the kernels' failure path: a
forward launch whose first copies are never issued (a test hook) must end by
itself with the error flag set, and the next launch on the same context must
be right."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def nvcc():
    for c in (shutil.which("nvcc"), os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not found")


def test_tensor_core_convolutions_match_float32_kernels(tmp_path):
    exe = str(tmp_path / "conv_tc_check")
    src = os.path.join(ROOT, "tests", "native", "conv_tc_check.cu")
    cmd = [nvcc(), "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "airboxcalc_gb300", "csrc"), "-o", exe, src]
    subprocess.run(cmd, check=True, capture_output=True, timeout=600)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "all match" in r.stdout
