"""The GB300 energy services driven through the C++ request interface
(Server -> work items in pinned buffers -> item processors -> C ABI), as a
reference caller would use them: results equal the direct C-ABI call."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from test_gpu_rigid import upload

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


@pytest.fixture(scope="module")
def shim(tmp_path_factory, pkg):
    from gbattract import _lib
    _lib.load()
    out = tmp_path_factory.mktemp("svc") / "libsvcshim.so"
    libdir = _lib.LIB_PATH.parent
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread",
                    str(HERE / "csrc" / "service_shim.cpp"), "-I", str(ROOT / "include"),
                    "-I", "/usr/local/cuda/include", "-L", str(libdir), "-lgbattract",
                    "-L", "/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{libdir}",
                    "-o", str(out)], check=True)
    return C.CDLL(str(out))


@pytest.fixture(scope="module")
def ctx(pkg):
    from gbattract.context import GbaContext
    c = GbaContext(0)
    yield c
    c.close()


@pytest.mark.parametrize("workers,item", [(1, 100), (2, 7), (4, 1000), (3, 1)])
def test_rigid_service_through_server(small_case, shim, ctx, workers, item):
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    want = ctx.energy_6d(*ids, wl.dofs)
    out = np.zeros((len(wl.dofs), 7), np.float32)
    err = C.create_string_buffer(512)
    rc = shim.run_service_6d(ctx.h, *[C.c_uint32(i) for i in ids], C.c_void_p(wl.dofs.ctypes.data),
                             C.c_size_t(len(wl.dofs)), workers, item, C.c_void_p(out.ctypes.data), err, 512)
    assert rc == 0, err.value
    assert np.array_equal(out, want)


def test_service_error_surfaces_in_wait(small_case, shim, ctx):
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    out = np.zeros((len(wl.dofs), 7), np.float32)
    err = C.create_string_buffer(512)
    rc = shim.run_service_6d(ctx.h, C.c_uint32(ids[0]), C.c_uint32(ids[1]), C.c_uint32(ids[2]),
                             C.c_uint32(424242), C.c_void_p(wl.dofs.ctypes.data),
                             C.c_size_t(len(wl.dofs)), 2, 16, C.c_void_p(out.ctypes.data), err, 512)
    assert rc == 1 and b"unknown parameter table id" in err.value


def test_modes_service_through_server(pkg, oracle, shim, ctx):
    wl = pkg.synth.make_pair(2, 100, 50, 40, (16.0, 23.0), n_modes=3, seed=616)
    opts = pkg.GridOptions()
    gr, gl = oracle.build_grid(wl.rec, wl.params, opts), oracle.build_grid(wl.lig, wl.params, opts)
    ids = (ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_grid(gr),
           ctx.upload_grid(gl), ctx.upload_params(wl.params))
    want = ctx.energy_6d_modes(*ids, wl.dofs)
    out = np.zeros((len(wl.dofs), 27), np.float32)
    err = C.create_string_buffer(512)
    rc = shim.run_service_6d_modes(ctx.h, *[C.c_uint32(i) for i in ids], C.c_void_p(wl.dofs.ctypes.data),
                                   C.c_size_t(len(wl.dofs)), 2, 9, C.c_void_p(out.ctypes.data), err, 512)
    assert rc == 0, err.value
    assert np.array_equal(out, want)
