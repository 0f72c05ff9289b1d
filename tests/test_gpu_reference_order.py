"""GBA_KOPT_REFERENCE_ORDER: the kernels sum every pose in the reference CPU
path's operation order (CPUEnergyService6D, src/service/CPUEnergyService6D.tpp:63-200:
bead by bead, grid term then the neighbour list in list order with the
reference's float and double steps, then the bead sums in bead order).

The device then equals the reference bit for bit wherever the reference's
sin/cos are correctly rounded:
* against the reference's own outputs (the golden fixtures) on every pose
  whose angles the generating host's sinf/cosf rounded correctly;
* against the oracle with correctly rounded sin/cos on every pose, at the
  sizes of config 0 and on a config-1 sample;
* minimization: config 0 in full (1,000 poses, maxFunEval 100) -- the
  device VA13 trajectories, evaluation counts and final results equal the
  oracle's minfor driving the same arithmetic, bit for bit, in the
  persistent kernel, the plain per-step form and a multi-pair batch.
With the host C library's sin/cos tabulated on the device as well
(gba_set_host_sincos) the device equals the oracle as the reference runs it
on this host -- libm sin/cos -- on every pose, minimizations included.
The normal-mode path (CPUEnergyService6DModes,
src/service/CPUEnergyService6DModes.tpp:121-327) likewise: the reference's
modes fixture, a config-2 sample, config-2 minimizations over 16 DOF.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu

KOPT_DEFAULT = 15
KOPT_REFERENCE_ORDER = 16
RIGID = ["rigid_synth", "rigid_const", "rigid_pdb"]


@pytest.fixture(scope="module")
def ctx(pkg):
    from gbattract.context import GbaContext
    c = GbaContext(0)
    c.set_kernel_options(KOPT_DEFAULT | KOPT_REFERENCE_ORDER)
    yield c
    c.close()


def _upload(ctx, rec, lig, grid, params):
    return (ctx.upload_protein(rec), ctx.upload_protein(lig), ctx.upload_grid(grid),
            ctx.upload_params(params))


@pytest.mark.parametrize("name", RIGID)
def test_equals_reference_outputs(name, golden_cases, oracle, ctx):
    d = golden_cases[name]
    rec, lig, params, opts = golden_inputs(d)
    grid = oracle.build_grid(rec, params, opts)
    ids = _upload(ctx, rec, lig, grid, params)
    got = ctx.energy_6d(*ids, d["dofs"])
    exact = d["sincos_exact"].astype(bool)
    with oracle.exact_sincos():
        ref_x = oracle.energy_6d(rec, lig, grid, params, d["dofs"])
    print(f"{name}: {int(exact.sum())}/{len(exact)} poses with correctly rounded libm sin/cos; "
          f"bitwise equal to the reference on {int(np.all(got == d['ref_out'], axis=1).sum())}")
    assert exact.mean() > 0.9
    assert np.array_equal(got[exact], d["ref_out"][exact])
    assert np.array_equal(got, ref_x)
    for i in ids:
        ctx.release(i)


def test_option_combinations_agree(small_case, oracle, ctx):
    """The order ignores the other options (it reads the ratio table and the
    native corners): every combination, with and without the octet copy,
    gives the same bits, equal to the exact-sincos oracle."""
    wl, grid = small_case
    ids = _upload(ctx, wl.rec, wl.lig, grid, wl.params)
    with oracle.exact_sincos():
        ref = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs)
    try:
        for flags, octets in ((16, False), (16 | 8, False), (31, True), (16 | 2, True)):
            ctx.grid_octets(ids[2], octets)
            ctx.set_kernel_options(flags)
            assert np.array_equal(ctx.energy_6d(*ids, wl.dofs), ref), flags
    finally:
        ctx.set_kernel_options(KOPT_DEFAULT | KOPT_REFERENCE_ORDER)
        ctx.grid_octets(ids[2], False)
    for i in ids:
        ctx.release(i)


def test_noalloc_and_batch_follow_the_option(small_case, oracle, ctx):
    import torch
    wl, grid = small_case
    ids = _upload(ctx, wl.rec, wl.lig, grid, wl.params)
    ref = ctx.energy_6d(*ids, wl.dofs)
    fn = ctx.lib.gba_energy_6d_noalloc
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t,
                   C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    d = torch.from_numpy(wl.dofs).cuda()
    out = torch.empty((len(wl.dofs), 7), dtype=torch.float32, device="cuda")
    assert fn(ctx.h, *ids, d.data_ptr(), len(wl.dofs), out.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    (be,) = ctx.batch_energy_6d([(*ids, wl.dofs)])
    assert np.array_equal(be, ref)
    for i in ids:
        ctx.release(i)


def test_config1_sample_bitwise(pkg, oracle, ctx):
    """Receptor 2000 / ligand 700 beads, 2,048 of config 1's poses, on the
    device-built grid with its octet copy."""
    wl = pkg.synth.make_config(1)
    dofs = np.ascontiguousarray(wl.dofs[:2048])
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gid = ctx.build_grid(rec, par, pkg.GridOptions())
    ctx.grid_octets(gid, True)
    host = ctx.download_grid(gid)
    got = ctx.energy_6d(rec, lig, gid, par, dofs)
    with oracle.exact_sincos():
        ref = oracle.energy_6d(wl.rec, wl.lig, host, wl.params, dofs)
    assert np.array_equal(got, ref)
    for i in (gid, lig, rec, par):
        ctx.release(i)


def test_config0_minimization_bitwise(pkg, oracle, ctx):
    wl = pkg.synth.make_config(0)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gid = ctx.build_grid(rec, par, pkg.GridOptions())
    ids = (rec, lig, gid, par)
    grid = ctx.download_grid(gid)
    steps = wl.steps
    dev = ctx.minimize_6d(*ids, wl.dofs, max_evals=steps)
    with oracle.exact_sincos():
        ref = oracle.minimize_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, steps)
    for a, b, what in zip(dev, ref, ("states", "results", "evaluations")):
        assert np.array_equal(a, b), what
    plain = ctx.minimize_6d_plain(*ids, wl.dofs[:200], max_evals=steps)
    for a, b in zip(plain, ref):
        assert np.array_equal(a, b[:200])
    # against the oracle as the reference runs it (the C library's sin/cos)
    _, r_libm, _ = oracle.minimize_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, steps)
    st = oracle.minimization_stats(dev[1], r_libm)
    same = float(np.mean(np.all(dev[1] == r_libm, axis=1)))
    print(f"config 0 minimization in the reference order: bitwise equal to the exact-sincos oracle on "
          f"all {len(wl.dofs)} poses; vs the libm oracle {st}, identical trajectories {same:.3f}")
    for i in (gid, lig, rec, par):
        ctx.release(i)


def test_batch_minimize_bitwise(pkg, oracle, ctx):
    """Three pairs of uneven sizes in one batch: each pose's trajectory equals
    the oracle's."""
    pairs, refs = [], []
    for k, (nr, nl, npz) in enumerate([(120, 50, 40), (200, 90, 7), (90, 140, 65)]):
        wl = pkg.synth.make_pair(4, nr, nl, npz, (18.0, 28.0), seed=3000 + k)
        grid = oracle.build_grid(wl.rec, wl.params, pkg.GridOptions())
        pairs.append((*_upload(ctx, wl.rec, wl.lig, grid, wl.params), wl.dofs))
        with oracle.exact_sincos():
            refs.append(oracle.minimize_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, 60))
    got = ctx.batch_minimize_6d(pairs, max_evals=60)
    for g, r in zip(got, refs):
        for a, b in zip(g, r):
            assert np.array_equal(a, b)


def test_host_sincos_reproduces_the_reference_on_this_host(pkg, oracle, ctx):
    """With the host C library's sin/cos tabulated (gba_set_host_sincos), the
    device takes the very values the reference takes on this host, so the
    reference order equals the oracle as the reference runs it -- libm
    sin/cos, no correction -- on every pose: a config-1 sample's energies
    and config 0's minimizations in full (all three outputs)."""
    import time
    t0 = time.perf_counter()
    # minimization trajectories reach angles beyond 100 rad: the whole
    # supported range
    ctx.set_host_sincos(4096.0)
    print(f"host sin/cos table: {time.perf_counter() - t0:.2f} s")
    try:
        wl = pkg.synth.make_config(1)
        dofs = np.ascontiguousarray(wl.dofs[:2048])
        rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
        gid = ctx.build_grid(rec, par, pkg.GridOptions())
        host = ctx.download_grid(gid)
        exact = oracle.libm_sincos_rounds_exactly(dofs[:, 3:6])
        assert not exact.all()        # the sample does meet misrounded angles
        assert np.array_equal(ctx.energy_6d(rec, lig, gid, par, dofs),
                              oracle.energy_6d(wl.rec, wl.lig, host, wl.params, dofs))
        for i in (gid, lig, rec, par):
            ctx.release(i)

        wl = pkg.synth.make_config(0)
        rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
        gid = ctx.build_grid(rec, par, pkg.GridOptions())
        host = ctx.download_grid(gid)
        dev = ctx.minimize_6d(rec, lig, gid, par, wl.dofs, max_evals=wl.steps)
        ref = oracle.minimize_6d(wl.rec, wl.lig, host, wl.params, wl.dofs, wl.steps)
        for a, b, what in zip(dev, ref, ("states", "results", "evaluations")):
            assert np.array_equal(a, b), what
        st = oracle.minimization_stats(dev[1], ref[1])
        print(f"config 0 minimization, reference order + host sin/cos vs the oracle (libm): {st}")
        assert st["within_tol"] == 1.0
        for i in (gid, lig, rec, par):
            ctx.release(i)
    finally:
        ctx.set_host_sincos(0)


def _modes_ids(ctx, pkg, wl, octets=False):
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gr = ctx.build_grid(rec, par, pkg.GridOptions())
    gl = ctx.build_grid(lig, par, pkg.GridOptions())
    for g in (gr, gl):
        ctx.grid_octets(g, octets)
    return (rec, lig, gr, gl, par), ctx.download_grid(gr), ctx.download_grid(gl)


def test_modes_equals_reference_outputs(golden_cases, oracle, ctx):
    """The modes fixture (the reference's CPUEnergyService6DModes outputs):
    bit for bit on every pose whose angles and negated angles the generating
    host's libm rounded correctly; the correctly-rounded oracle on all."""
    d = golden_cases["modes_synth"]
    rec, lig, params, opts = golden_inputs(d)
    gr, gl = oracle.build_grid(rec, params, opts), oracle.build_grid(lig, params, opts)
    ids = (ctx.upload_protein(rec), ctx.upload_protein(lig), ctx.upload_grid(gr), ctx.upload_grid(gl),
           ctx.upload_params(params))
    got = ctx.energy_6d_modes(*ids, d["dofs"])
    exact = d["sincos_exact"].astype(bool)
    with oracle.exact_sincos():
        ref_x = oracle.energy_6d_modes(rec, lig, gr, gl, params, d["dofs"])
    assert np.array_equal(got[exact], d["ref_out"][exact])
    assert np.array_equal(got, ref_x)
    for i in ids:
        ctx.release(i)


def test_modes_config2_sample_bitwise(pkg, oracle, ctx):
    """Receptor 1500 / ligand 600 beads with 5 + 5 modes, 256 of config 2's
    poses, device-built grids with their octet copies."""
    wl = pkg.synth.make_config(2, n_poses=256)
    ids, hr, hl = _modes_ids(ctx, pkg, wl, octets=True)
    got = ctx.energy_6d_modes(*ids, wl.dofs)
    with oracle.exact_sincos():
        ref = oracle.energy_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs)
    assert np.array_equal(got, ref, equal_nan=True)
    for i in ids:
        ctx.release(i)


def test_modes_minimization_bitwise(pkg, oracle, ctx):
    """Config 2's modes minimization (16 DOF, maxFunEval 200) on 64 of its
    poses: device and plain forms equal the correctly-rounded oracle's VA13
    bit for bit; with the host's sin/cos tabulated, the oracle as the
    reference runs it."""
    wl = pkg.synth.make_config(2, n_poses=64)
    ids, hr, hl = _modes_ids(ctx, pkg, wl)
    dev = ctx.minimize_6d_modes(*ids, wl.dofs, max_evals=200)
    plain = ctx.minimize_6d_modes_plain(*ids, wl.dofs, max_evals=200)
    with oracle.exact_sincos():
        ref = oracle.minimize_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs, 200)
    for a, b, c in zip(dev, plain, ref):
        assert np.array_equal(a, c, equal_nan=True)
        assert np.array_equal(b, c, equal_nan=True)
    ctx.set_host_sincos(4096.0)
    try:
        dev = ctx.minimize_6d_modes(*ids, wl.dofs, max_evals=200)
    finally:
        ctx.set_host_sincos(0)
    ref = oracle.minimize_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs, 200)
    for a, c in zip(dev, ref):
        assert np.array_equal(a, c, equal_nan=True)
    st = oracle.minimization_stats(dev[1], ref[1])
    print(f"config 2 minimization sample, reference order + host sin/cos vs the oracle (libm): {st}")
    for i in ids:
        ctx.release(i)


def test_host_sincos_arguments(ctx):
    """Negative, NaN and too-wide ranges are refused; 0 turns the table off."""
    from gbattract._lib import GbaError
    for bad in (-1.0, 5000.0, float("nan")):
        with pytest.raises(GbaError):
            ctx.set_host_sincos(bad)
    ctx.set_host_sincos(0)


def test_team_sizes_in_the_reference_order(pkg, oracle, ctx):
    """Teams of 2..7 warps per pose (each warp a share of the ligand's 64-bead
    rounds, the bead totals added in round and bead order by the team's
    first warp) follow the oracle's trajectories bit for bit, as one warp
    does.  A 260-bead ligand has five rounds: teams of 2, 3 and 4 split
    unevenly."""
    wl = pkg.synth.make_pair(0, 500, 260, 300, (38.0, 46.0), seed=4242)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    gid = ctx.build_grid(rec, par, pkg.GridOptions())
    ids = (rec, lig, gid, par)
    grid = ctx.download_grid(gid)
    with oracle.exact_sincos():
        ref = oracle.minimize_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, 40)
    try:
        for team in (1, 2, 3, 4, 5, 7, 0):
            ctx.set_minimize_team(team)
            got = ctx.minimize_6d(*ids, wl.dofs, max_evals=40)
            for a, b in zip(got, ref):
                assert np.array_equal(a, b), f"team {team}"
    finally:
        ctx.set_minimize_team(0)
    for i in (gid, lig, rec, par):
        ctx.release(i)


@pytest.mark.parametrize("potshape,dielec", [(0, 0), (0, 1), (1, 1)])
def test_force_field_branches(pkg, oracle, ctx, potshape, dielec):
    """The 12-6 shape, both dielectrics and ipon in {-1, 0, 1, 2} (the
    synthetic tables use 8-6 and ipon 1): the reference order equals the
    correctly-rounded oracle bit for bit, the default order stays within the
    parity bound."""
    from test_gpu_rigid import pose_errors
    wl = pkg.synth.make_pair(0, 160, 70, 160, (15.0, 24.0), seed=9191)
    rng = np.random.default_rng(5)
    T = wl.params.num_types
    r0 = rng.uniform(3.0, 5.0, (T, T)).astype(np.float32)
    eps = rng.uniform(0.1, 10.0, (T, T)).astype(np.float32)
    ipon = rng.choice(np.array([-1, 0, 1, 2], np.int32), size=(T, T))
    wl.params.table = pkg.model.attract_params(r0, eps, ipon, potshape)
    wl.params.potshape = potshape
    wl.params.dielec = dielec
    grid = oracle.build_grid(wl.rec, wl.params, pkg.GridOptions())
    ids = _upload(ctx, wl.rec, wl.lig, grid, wl.params)
    with oracle.exact_sincos():
        ref_x, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    assert st["n_pairs"].sum() > 1000
    assert np.array_equal(ctx.energy_6d(*ids, wl.dofs), ref_x)
    try:
        ctx.set_kernel_options(KOPT_DEFAULT)
        got = ctx.energy_6d(*ids, wl.dofs)
    finally:
        ctx.set_kernel_options(KOPT_DEFAULT | KOPT_REFERENCE_ORDER)
    for e in pose_errors(got, ref_x, st):
        assert float(e.max()) <= 1e-4
    for i in ids:
        ctx.release(i)


@pytest.mark.parametrize("n_lig", [1, 63, 64, 65, 129])
def test_round_boundaries_and_edge_poses(pkg, oracle, ctx, n_lig):
    """Ligands of one, exactly full and partially filled 64-bead rounds, with
    non-finite and far-away poses mixed in: bit for bit the oracle's, NaN
    results included."""
    wl = pkg.synth.make_pair(0, 140, n_lig, 64, (12.0, 22.0), seed=300 + n_lig)
    dofs = wl.dofs.copy()
    dofs[5, 0] = np.nan
    dofs[9, 4] = np.inf
    dofs[13] = [500.0, 0.0, 0.0, 0.3, 0.2, 0.1]
    grid = oracle.build_grid(wl.rec, wl.params, pkg.GridOptions())
    ids = _upload(ctx, wl.rec, wl.lig, grid, wl.params)
    got = ctx.energy_6d(*ids, dofs)
    with oracle.exact_sincos():
        ref = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, dofs)
    assert np.array_equal(got, ref, equal_nan=True)
    for i in ids:
        ctx.release(i)


def test_modes_ten_mode_capacity(pkg, oracle, ctx):
    """Eight modes per protein (the kernels compiled for ten): scoring and a
    short minimization equal the correctly-rounded oracle bit for bit."""
    wl = pkg.synth.make_pair(2, 120, 60, 48, (16.0, 24.0), n_modes=8, seed=826)
    ids, hr, hl = _modes_ids(ctx, pkg, wl)
    got = ctx.energy_6d_modes(*ids, wl.dofs)
    with oracle.exact_sincos():
        ref = oracle.energy_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs)
        mref = oracle.minimize_6d_modes(wl.rec, wl.lig, hr, hl, wl.params, wl.dofs[:16], 40)
    assert np.array_equal(got, ref, equal_nan=True)
    for a, b in zip(ctx.minimize_6d_modes(*ids, wl.dofs[:16], max_evals=40), mref):
        assert np.array_equal(a, b, equal_nan=True)
    for i in ids:
        ctx.release(i)
