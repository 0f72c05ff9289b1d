"""The device grid builder (gba_build_grid) against the CPU oracle's builder.

Both builders perform the same IEEE-rounded FP32 operations per receptor bead
and sum in the same order (FP32 partials over blocks of 256 beads, added in
double), so the potentials must agree bit for bit; the neighbour lists are
tested in unfused double on both sides and must agree bit for bit too.  The
layout is that of readGridFromGridFile (src/fileIO/readFile.cpp:261-422):
channel 0 = charge, outer spacing 2x the inner with its origin derived from
the float inner origin, 0-based neighbour indices into the receptor; the
neighbour semantics are NLGrid's (src/model/NLGrid.tpp:29-51,
src/model/NLGrid.h:100-108).

The small pair and config 0's 500-bead receptor are compared in full.  For
config 1's 2,000-bead receptor (a 95x96x94 inner grid, 33 channels) the CPU
builder needs minutes, so the neighbour grid and list are compared in full
and the potentials on two whole z-slices plus 4,096 seeded random voxels of
each grid.  Finally the energies of config 0's 1,000 poses computed on the
device-built grid match the oracle's on the same grid (the energy parity
bound), so the benchmarked path's grids are pinned."""
import numpy as np
import pytest

from test_gpu_rigid import pose_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(pkg):
    from gbattract.context import GbaContext
    c = GbaContext(0)
    yield c
    c.close()


def _device_grid(ctx, wl, opts):
    rec, par = ctx.upload_protein(wl.rec), ctx.upload_params(wl.params)
    gid = ctx.build_grid(rec, par, opts)
    got = ctx.download_grid(gid)
    return got, (rec, par, gid)


def _same_desc(a, b):
    assert a.numGrids == b.numGrids
    assert tuple(a.dimN) == tuple(b.dimN)
    assert np.float32(a.gridSpacing) == np.float32(b.gridSpacing)
    assert np.array_equal(np.float32(a.posMin), np.float32(b.posMin))


def _same_nl(got, nl, ng, lst):
    assert tuple(got.nl.dimN) == tuple(nl.dimN) and got.nl.numEl == nl.numEl
    assert np.float32(got.nl.dPlateau) == np.float32(nl.dPlateau)
    assert np.array_equal(np.float32(got.nl.posMin), np.float32(nl.posMin))
    assert np.array_equal(got.nl_grid, ng)
    assert np.array_equal(got.nl_list, lst)


@pytest.mark.parametrize("which", ["small", "config0"])
def test_device_builder_bitwise(pkg, oracle, ctx, which):
    if which == "small":
        wl = pkg.synth.make_pair(0, 150, 60, 8, (18.0, 26.0), seed=11)
    else:
        wl = pkg.synth.make_config(0, n_poses=8)
    opts = pkg.GridOptions()
    got, ids = _device_grid(ctx, wl, opts)
    want = oracle.build_grid(wl.rec, wl.params, opts)
    _same_desc(got.inner, want.inner)
    _same_desc(got.outer, want.outer)
    assert np.array_equal(got.inner_data.view(np.uint32), want.inner_data.view(np.uint32))
    assert np.array_equal(got.outer_data.view(np.uint32), want.outer_data.view(np.uint32))
    _same_nl(got, want.nl, want.nl_grid, want.nl_list)
    # non-trivial content: every channel has non-zero potential, lists are long
    assert np.all(np.abs(got.inner_data[..., 3]).reshape(got.inner.numGrids, -1).max(axis=1) > 0)
    assert want.nl.numEl > 100 * wl.rec.n
    for i in ids:
        ctx.release(i)


def test_device_builder_config1_lists_and_voxels(pkg, oracle, ctx):
    wl = pkg.synth.make_config(1, n_poses=8)
    opts = pkg.GridOptions()
    got, ids = _device_grid(ctx, wl, opts)
    inner, outer, _ = oracle.grid_layout(wl.rec, opts)
    _same_desc(got.inner, inner)
    _same_desc(got.outer, outer)
    nl, ng, lst = oracle.build_grid_nl(wl.rec, opts)
    _same_nl(got, nl, ng, lst)
    rng = np.random.default_rng(2024)
    for desc, data in ((got.inner, got.inner_data), (got.outer, got.outer_data)):
        Nx, Ny, Nz = desc.dimN
        plane = Nx * Ny
        slices = [np.arange(z * plane, (z + 1) * plane) for z in (Nz // 2, Nz // 3)]
        vox = np.unique(np.concatenate(slices + [rng.choice(desc.nvox, 4096, replace=False)]))
        want = oracle.grid_voxels(wl.rec, wl.params, opts, desc, vox)
        have = data.reshape(desc.numGrids, -1, 4)[:, vox, :].transpose(1, 0, 2)
        assert np.array_equal(have.view(np.uint32), want.view(np.uint32))
    for i in ids:
        ctx.release(i)


def test_energy_on_device_built_grid(pkg, oracle, ctx):
    """Config 0 in full (500/200 beads, 1,000 poses) scored on the grid the
    device built, against the oracle scoring the same grid."""
    wl = pkg.synth.make_config(0)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gid = ctx.build_grid(rec, par, pkg.GridOptions())
    ctx.grid_octets(gid, True)       # the bench's default layout
    host = ctx.download_grid(gid)
    got = ctx.energy_6d(rec, lig, gid, par, wl.dofs)
    ref, st = oracle.energy_6d(wl.rec, wl.lig, host, wl.params, wl.dofs, stats=True)
    for e in pose_errors(got, ref, st):
        assert float(e.max()) <= 1e-4
    cen, _ = ctx.census_6d(rec, lig, gid, par, wl.dofs)
    assert np.array_equal(cen[:, 0], st["n_grid"]) and np.array_equal(cen[:, 3], st["n_nl_entries"])
    for i in (gid, lig, rec, par):
        ctx.release(i)
