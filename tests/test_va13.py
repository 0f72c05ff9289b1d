"""The library's resumable VA13 (va13.cuh, used by the device minimizer and
the plain driver) against the oracle's literal restatement of minfor.f /
mc11a.f: identical evaluation sequences, bit for bit, on an analytic function."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = tmp_path_factory.mktemp("va13") / "libva13trace.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    str(HERE / "csrc" / "va13_trace.cpp"), "-o", str(out)], check=True)
    return C.CDLL(str(out))


@pytest.mark.parametrize("n,ivmax,seed", [(6, 500, 0), (6, 40, 1), (16, 300, 2), (2, 200, 3)])
def test_va13_matches_minfor(harness, oracle, n, ivmax, seed):
    x0 = np.random.default_rng(seed).uniform(-1.5, 1.5, n)
    cap = ivmax + 2
    a = np.zeros(cap * (n + 1))
    b = np.zeros(cap * (n + 1))
    lib = oracle.lib()
    lib.orc_minfor_trace.restype = C.c_int
    ka = lib.orc_minfor_trace(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(a.ctypes.data), cap)
    kb = harness.va13_trace(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(b.ctypes.data), cap)
    assert ka == kb and ka > 1
    assert ka <= ivmax + 1
    assert np.array_equal(a[: ka * (n + 1)], b[: kb * (n + 1)])
    # the minimizer makes progress on Rosenbrock
    fa = a[: ka * (n + 1)].reshape(ka, n + 1)[:, n]
    assert fa.min() < fa[0]


@pytest.mark.parametrize("nan_eval", [0, 2, 7])
def test_va13_matches_minfor_on_nan_gradients(harness, oracle, nan_eval):
    """A NaN gradient component (an energy that overflowed) sends both
    implementations down the same branches: max, min and abs follow the C++
    library's semantics in each."""
    n, ivmax = 6, 60
    x0 = np.random.default_rng(11).uniform(-1.5, 1.5, n)
    cap = ivmax + 2
    a = np.zeros(cap * (n + 1))
    b = np.zeros(cap * (n + 1))
    lib = oracle.lib()
    lib.orc_minfor_trace_nan.restype = C.c_int
    ka = lib.orc_minfor_trace_nan(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(a.ctypes.data), cap,
                                  nan_eval)
    kb = harness.va13_trace_nan(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(b.ctypes.data), cap,
                                nan_eval)
    assert ka == kb and ka > nan_eval
    assert np.array_equal(a[: ka * (n + 1)], b[: kb * (n + 1)], equal_nan=True)
