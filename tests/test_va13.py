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


def _form_trace(harness, n, x0, ivmax, nan_eval, kind, warp):
    cap = ivmax + 2
    out = np.zeros(cap * (n + 1))
    k = harness.va13_trace_form(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(out.ctypes.data), cap,
                                nan_eval, kind, warp)
    assert k > 0
    return out[: k * (n + 1)].reshape(k, n + 1)


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [2, 6, 16, 26, 31])
def test_warp_form_matches_machine(harness, kind, n):
    """The warp form (provide_w, used by the device minimizers: element-wise
    updates on lanes, independent divisions together), run here with the
    elements of each section in descending order, takes the machine's
    trajectory bit for bit on several objectives, with and without a NaN
    gradient."""
    for seed in range(3):
        x0 = np.random.default_rng(100 * n + seed).uniform(-1.5, 1.5, n)
        for nan_eval in (-1, 3):
            a = _form_trace(harness, n, x0, 300, nan_eval, kind, 0)
            b = _form_trace(harness, n, x0, 300, nan_eval, kind, 1)
            assert a.shape == b.shape
            assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("n", [6, 16])
def test_warp_form_matches_minfor(harness, oracle, n):
    x0 = np.random.default_rng(7 + n).uniform(-1.5, 1.5, n)
    ivmax = 300
    cap = ivmax + 2
    a = np.zeros(cap * (n + 1))
    lib = oracle.lib()
    lib.orc_minfor_trace.restype = C.c_int
    ka = lib.orc_minfor_trace(n, C.c_void_p(x0.ctypes.data), ivmax, C.c_void_p(a.ctypes.data), cap)
    b = _form_trace(harness, n, x0, ivmax, -1, 0, 1)
    assert b.shape[0] == ka
    assert np.array_equal(a[: ka * (n + 1)], b.ravel())


def test_update_forms_on_arbitrary_inputs(harness):
    """mc11a and mc11e against their warp forms on random factors, vectors,
    sig, ir, mk and eps -- every path of mc11a, including those minfor never
    takes (ir > 0 on entry, eps != 0, z passed as w)."""
    f = harness.va13_update_forms
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_double,
                  C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(0)
    for _ in range(6000):
        n = int(rng.choice([1, 2, 3, 6, 16, 26, 31]))
        na = n * (n + 1) // 2
        a = rng.normal(0, 1, na)
        k = 0
        for i in range(n):   # diagonal: mostly positive, some zero or negative
            u = rng.random()
            a[k] = abs(a[k]) + 0.1 if u < 0.8 else (0.0 if u < 0.9 else -abs(a[k]))
            k += n - i
        z, w = rng.normal(0, 1, n), rng.normal(0, 1, n)
        if rng.random() < 0.1:
            z[rng.integers(n)] = 0.0
        sig = float(rng.choice([-1.0, 1.0, 0.0])) * float(rng.lognormal(0, 2))
        o1 = np.zeros(na + 2 * n + 1)
        o2 = np.zeros_like(o1)
        f(n, a.ctypes.data, z.ctypes.data, w.ctypes.data, sig, int(rng.integers(-n - 1, n + 2)),
          int(rng.integers(0, 2)), float(rng.choice([0.0, 1e-3, 0.5])), int(rng.random() < 0.3),
          int(rng.random() < 0.3), o1.ctypes.data, o2.ctypes.data)
        assert np.array_equal(o1, o2, equal_nan=True)
