"""The VA13 machine's warp form on the GPU -- one warp, element j on lane j,
the form the device minimizers step -- against the host machine bit for bit,
on objectives that evaluate to the same bits on both sides
(tests/csrc/va13_objectives.h), with n up to 31 and NaN gradients.  The
minimizer tests cover the same code through the energy kernels at n = 6 and
6 + modes; this one reaches every branch the machine takes on the analytic
objectives, at every lane count."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def libs(tmp_path_factory):
    d = tmp_path_factory.mktemp("va13dev")
    host, dev = d / "libva13trace.so", d / "libva13dev.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    str(HERE / "csrc" / "va13_trace.cpp"), "-o", str(host)], check=True)
    nvcc = "/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else "nvcc"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "--expt-relaxed-constexpr", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
                    str(HERE / "csrc" / "va13_warp_device.cu"), "-o", str(dev)], check=True)
    return C.CDLL(str(host)), C.CDLL(str(dev))


@pytest.mark.parametrize("kind", [0, 1, 4, 5])
@pytest.mark.parametrize("n", [6, 16, 26, 31])
def test_device_warp_form_matches_host_machine(libs, kind, n):
    host, dev = libs
    ivmax = 300
    cap = ivmax + 2
    for seed in range(2):
        x0 = np.random.default_rng(1000 * kind + 10 * n + seed).uniform(-1.5, 1.5, n)
        for nan_eval in (-1, 3):
            a = np.zeros(cap * (n + 1))
            b = np.zeros(cap * (n + 1))
            ka = host.va13_trace_form(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(a.ctypes.data), cap,
                                      nan_eval, kind, 0)
            kb = dev.va13_device_trace(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(b.ctypes.data), cap,
                                       nan_eval, kind)
            assert ka > 0 and kb == ka, (seed, nan_eval, ka, kb)
            assert np.array_equal(a[: ka * (n + 1)], b[: kb * (n + 1)], equal_nan=True), (seed, nan_eval)
