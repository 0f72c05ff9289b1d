"""gba_energy_6d_noalloc through the C ABI: the scoring call for callers that
must not allocate device memory while they score (a service under a fixed
memory budget, a host that reserved the device's memory up front).  Its
scratch is a static device array; its results must equal gba_energy_6d's.

Named to be collected last, so that it runs both after the other GPU tests
and alone (pytest tests/test_zz_no_alloc.py)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fn(lib):
    fn = lib.gba_energy_6d_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t,
                   C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def allocations(lib) -> int:
    v = C.c_uint64()
    assert lib.gba_allocation_count(C.byref(v)) == 0
    return v.value


@pytest.fixture(scope="module")
def setup(pkg):
    import torch
    from gbattract import _lib
    from gbattract.context import GbaContext
    lib = _lib.load()
    ctx = GbaContext(0)
    wl = pkg.synth.make_pair(1, 500, 200, 5000, (35.0, 45.0), seed=5150)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    grid = ctx.build_grid(rec, par, pkg.GridOptions())
    dofs = torch.from_numpy(wl.dofs).cuda()
    yield ctx, _fn(lib), (rec, lig, grid, par), dofs
    ctx.close()


def call(ctx, fn, ids, dofs, n, out):
    return fn(ctx.h, *ids, C.c_void_p(dofs.data_ptr()), n, C.c_void_p(out.data_ptr()), None)


@pytest.mark.parametrize("n", [5000, 100])
def test_two_calls_match_energy_6d(setup, n):
    import torch
    ctx, fn, ids, dofs = setup
    d = dofs[:n].contiguous()
    want = ctx.energy_6d(*ids, d)            # existing entry point (stream-ordered scratch)
    torch.cuda.synchronize()
    outs = []
    for _ in range(2):
        out = torch.full((n, 7), float("nan"), dtype=torch.float32, device="cuda")
        assert call(ctx, fn, ids, d, n, out) == 0, ctx.lib.gba_last_error(ctx.h)
        torch.cuda.synchronize()
        outs.append(out)
    assert torch.equal(outs[0], want) and torch.equal(outs[1], want)


def test_first_call_on_fresh_context_allocates_nothing(pkg):
    """The entry point's first calls on a new context and new data ids, before
    any other scoring call, make no allocation (the library's own count) and
    take no device memory; gba_energy_6d afterwards gives the same bits."""
    import torch
    from gbattract import _lib
    from gbattract.context import GbaContext
    lib = _lib.load()
    fn = _fn(lib)
    wl = pkg.synth.make_pair(1, 400, 150, 6000, (33.0, 43.0), seed=6161)
    with GbaContext(0) as ctx:
        rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
        grid = ctx.build_grid(rec, par, pkg.GridOptions())
        ids = (rec, lig, grid, par)
        dofs = torch.from_numpy(wl.dofs).cuda()
        outs = [torch.full((len(wl.dofs), 7), float("nan"), dtype=torch.float32, device="cuda")
                for _ in range(2)]
        torch.cuda.synchronize()
        count0 = allocations(lib)
        free0, _ = torch.cuda.mem_get_info()
        for out in outs:
            assert call(ctx, fn, ids, dofs, len(wl.dofs), out) == 0, ctx.lib.gba_last_error(ctx.h)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert allocations(lib) == count0
        assert free1 >= free0
        want = ctx.energy_6d(*ids, dofs)
        assert torch.equal(outs[0], want) and torch.equal(outs[1], want)


def test_oversize_batch_rejected(setup):
    import torch
    ctx, fn, ids, dofs = setup
    n = 65537
    big = torch.zeros((n, 6), dtype=torch.float32, device="cuda")
    out = torch.empty((n, 7), dtype=torch.float32, device="cuda")
    assert call(ctx, fn, ids, big, n, out) == 1
    assert b"static scratch limit" in ctx.lib.gba_last_error(ctx.h)
    host = np.zeros((10, 6), np.float32)
    rc = fn(ctx.h, *ids, C.c_void_p(host.ctypes.data), 10, C.c_void_p(out.data_ptr()), None)
    assert rc == 1 and b"device pointers" in ctx.lib.gba_last_error(ctx.h)
