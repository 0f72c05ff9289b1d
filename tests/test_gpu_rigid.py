"""Parity of the fused rigid kernel (through the C ABI) with the reference
CPU path: golden fixtures of the reference's own outputs, the oracle on fresh
seeded cases, bit-exact census counts, the host- and device-pointer paths and
the error behaviour.

Tolerance: per pose, |got - ref| / max(|ref|, 0.05 * S) <= 1e-4 for the energy
and for the force and torque vectors (Euclidean norms), where S is the sum of
absolute term magnitudes the oracle reports for that pose.  The floor bounds
the FP32 summation error of heavily cancelling sums (~sqrt(n) * 6e-8 * S)."""
import numpy as np
import pytest

from conftest import golden_inputs

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def pose_errors(got, ref, st):
    got = got.astype(np.float64)
    ref = ref.astype(np.float64)
    eE = np.abs(got[:, 0] - ref[:, 0]) / np.maximum(np.abs(ref[:, 0]), 0.05 * st["abs_E"] + 1e-30)
    eF = np.linalg.norm(got[:, 1:4] - ref[:, 1:4], axis=1) / np.maximum(
        np.linalg.norm(ref[:, 1:4], axis=1), 0.05 * st["abs_F"] + 1e-30)
    eT = np.linalg.norm(got[:, 4:7] - ref[:, 4:7], axis=1) / np.maximum(
        np.linalg.norm(ref[:, 4:7], axis=1), 0.05 * st["abs_T"] + 1e-30)
    return eE, eF, eT


@pytest.fixture(scope="module")
def ctx(pkg):
    from gbattract.context import GbaContext
    c = GbaContext(0)
    yield c
    c.close()


def upload(ctx, rec, lig, grid, params):
    return (ctx.upload_protein(rec), ctx.upload_protein(lig), ctx.upload_grid(grid),
            ctx.upload_params(params))


@pytest.mark.parametrize("name", ["rigid_synth", "rigid_const", "rigid_pdb"])
def test_golden_reference_outputs(name, golden_cases, oracle, ctx):
    d = golden_cases[name]
    rec, lig, params, opts = golden_inputs(d)
    grid = oracle.build_grid(rec, params, opts)
    _, st = oracle.energy_6d(rec, lig, grid, params, d["dofs"], stats=True)
    got = ctx.energy_6d(*upload(ctx, rec, lig, grid, params), d["dofs"])
    for e in pose_errors(got, d["ref_out"], st):
        assert float(e.max()) <= RTOL


def test_fresh_case_vs_oracle_and_census(small_case, oracle, ctx):
    wl, grid = small_case
    ref, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    got = ctx.energy_6d(*ids, wl.dofs)
    for e in pose_errors(got, ref, st):
        assert float(e.max()) <= RTOL
    cen, res2 = ctx.census_6d(*ids, wl.dofs)
    # grid indices and neighbour walks are bit-exact: identical counts per pose
    assert np.array_equal(cen[:, 0], st["n_grid"])
    assert np.array_equal(cen[:, 1], st["n_grid_charged"])
    assert np.array_equal(cen[:, 2], st["n_nl"])
    assert np.array_equal(cen[:, 3], st["n_nl_entries"])
    assert np.array_equal(res2, got)


def test_device_and_host_pointers_agree(small_case, ctx):
    import torch
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    host = ctx.energy_6d(*ids, wl.dofs)
    d = torch.from_numpy(wl.dofs).cuda()
    dev = ctx.energy_6d(*ids, d)
    torch.cuda.synchronize()
    assert dev.is_cuda
    assert np.array_equal(dev.cpu().numpy(), host)
    pinned = torch.from_numpy(wl.dofs).pin_memory()
    pin_out = ctx.energy_6d(*ids, pinned)
    assert np.array_equal(pin_out.numpy(), host)


def test_edge_sizes(small_case, oracle, ctx):
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    empty = ctx.energy_6d(*ids, np.zeros((0, 6), np.float32))
    assert empty.shape == (0, 7)
    one = ctx.energy_6d(*ids, wl.dofs[:1])
    ref = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs[:1])
    assert np.allclose(one, ref, rtol=1e-4, atol=1e-3 * np.abs(ref).max())
    # a pose far outside every grid interacts with nothing
    far = np.array([[500.0, 0, 0, 0.3, 0.2, 0.1]], np.float32)
    assert np.all(ctx.energy_6d(*ids, far) == 0.0)
    # odd pose counts that do not fill a warp / block / wave
    for n in (31, 33, 257):
        dofs = np.repeat(wl.dofs, (n + len(wl.dofs) - 1) // len(wl.dofs), axis=0)[:n]
        out = ctx.energy_6d(*ids, dofs)
        assert np.array_equal(out[: len(wl.dofs)], ctx.energy_6d(*ids, dofs[: len(wl.dofs)]))


@pytest.mark.parametrize("n_lig", [1, 63, 64, 65, 129])
def test_ligand_round_boundaries(pkg, oracle, ctx, n_lig):
    """Ligands of 1, 63, 64, 65 and 129 beads: one, exactly full and
    partially filled rounds of 64 staged beads, against the oracle."""
    wl = pkg.synth.make_pair(0, 140, n_lig, 64, (12.0, 22.0), seed=300 + n_lig)
    grid = oracle.build_grid(wl.rec, wl.params, pkg.GridOptions())
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    got = ctx.energy_6d(*ids, wl.dofs)
    ref, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    for e in pose_errors(got, ref, st):
        assert float(e.max()) <= RTOL
    cen, _ = ctx.census_6d(*ids, wl.dofs)
    for col, key in enumerate(("n_grid", "n_grid_charged", "n_nl", "n_nl_entries")):
        assert np.array_equal(cen[:, col], st[key])


def test_non_finite_poses_leave_the_others_alone(small_case, ctx):
    """Poses with NaN or infinite translations or angles fail every grid and
    neighbour-list bounds test, so they touch no grid memory and score zero
    energy and force; the finite poses of the same batch keep their results
    bit for bit (also through the visiting-order pass, which sends NaN keys
    to cell 0)."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    clean = ctx.energy_6d(*ids, wl.dofs)
    bad = wl.dofs.copy()
    rows = np.arange(0, len(bad), 3)
    bad[rows[0::4], 0] = np.nan
    bad[rows[1::4], 1] = np.inf
    bad[rows[2::4], 3] = np.nan
    bad[rows[3::4], 2] = -np.inf
    keep = np.setdiff1d(np.arange(len(bad)), rows)
    for n_rep in (1, 80):          # the second batch is large enough to be visiting-ordered
        d = np.tile(bad, (n_rep, 1))
        out = ctx.energy_6d(*ids, d)
        for r in range(n_rep):
            o = out[r * len(bad):(r + 1) * len(bad)]
            assert np.array_equal(o[keep], clean[keep])
            assert np.all(o[rows, :4] == 0.0)


def test_pose_order_does_not_change_results(small_case, ctx):
    """Large batches are visited grouped by translation; every pose keeps its slot."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    rng = np.random.default_rng(8)
    dofs = wl.dofs[rng.integers(0, len(wl.dofs), 6000)]
    dofs[:, :3] += rng.normal(0, 3.0, (6000, 3)).astype(np.float32)
    ctx.set_pose_order(False)
    plain = ctx.energy_6d(*ids, dofs)
    ctx.set_pose_order(True)
    ordered = ctx.energy_6d(*ids, dofs)
    assert np.array_equal(plain, ordered)


@pytest.mark.parametrize("n", [1, 31, 4863, 4865, 9731])
def test_pose_counter_visits_every_pose_once(small_case, ctx, n):
    """Warps claim poses from a per-launch counter: every pose of a batch is
    evaluated exactly once and lands in its own slot, whatever the batch size
    relative to the resident warps, and equals the same pose scored in small
    batches (other launch shapes, fewer poses than warps)."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    rng = np.random.default_rng(n)
    dofs = wl.dofs[rng.integers(0, len(wl.dofs), n)]
    dofs[:, :3] += rng.normal(0, 3.0, (n, 3)).astype(np.float32)
    whole = ctx.energy_6d(*ids, dofs)
    pieces = np.concatenate([ctx.energy_6d(*ids, dofs[k:k + 97]) for k in range(0, n, 97)])
    assert np.array_equal(whole, pieces)


def test_octet_layout_does_not_change_results(small_case, ctx):
    """The duplicated-octet layout reads the same corners: with one lane per
    lookup the results are bit-identical to the native layout.  (The 8-lane
    cooperative lookup, default on octet grids, sums the same per-lookup
    values on other lanes; it is held to the parity bound in
    test_kernel_options_keep_parity.)"""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    try:
        ctx.set_kernel_options(1 | 4)       # computed ratio, four blocks; no cooperative lookup
        native = ctx.energy_6d(*ids, wl.dofs)
        ctx.grid_octets(ids[2], True)
        octets = ctx.energy_6d(*ids, wl.dofs)
        s1, r1, n1 = ctx.minimize_6d(*ids, wl.dofs[:32], max_evals=30)
        ctx.grid_octets(ids[2], False)
        s2, r2, n2 = ctx.minimize_6d(*ids, wl.dofs[:32], max_evals=30)
    finally:
        ctx.set_kernel_options(15)
        ctx.grid_octets(ids[2], False)
    assert np.array_equal(native, octets)
    assert np.array_equal(r1, r2) and np.array_equal(s1, s2)


def test_typed_list_is_bitwise_the_gather(small_case, pkg, ctx):
    """GBA_KOPT_TYPED_LIST reads the receptor type from a per-receptor copy of
    the neighbour list: results are bit-identical to gathering the type per
    pair, for scoring and minimization, and the copies are kept per receptor
    (a second receptor on the same grid gets its own)."""
    wl, grid = small_case
    rec, lig, g, p = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    moved = pkg.Protein(xyz=wl.rec.xyz + np.float32(0.37), type=wl.rec.type,
                        mapped=wl.rec.mapped, charge=wl.rec.charge[::-1].copy())
    rec2 = ctx.upload_protein(moved)
    out = {}
    try:
        for flags in (7, 15):
            ctx.set_kernel_options(flags)
            out[flags] = (ctx.energy_6d(rec, lig, g, p, wl.dofs),
                          ctx.energy_6d(rec2, lig, g, p, wl.dofs),
                          ctx.minimize_6d(rec, lig, g, p, wl.dofs[:16], max_evals=30)[1])
        ctx.release(rec2)
        again = ctx.energy_6d(rec, lig, g, p, wl.dofs)
    finally:
        ctx.set_kernel_options(15)
    for a, b in zip(out[7], out[15]):
        assert np.array_equal(a, b)
    assert not np.array_equal(out[15][0], out[15][1])
    assert np.array_equal(again, out[15][0])


def test_errors(small_case, pkg, ctx):
    from gbattract import GbaError
    wl, grid = small_case
    rec, lig, g, p = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    with pytest.raises(GbaError) as e:
        ctx.energy_6d(rec, lig, g, 9999, wl.dofs)
    assert e.value.code == 2
    with pytest.raises(GbaError) as e:
        ctx.energy_6d(rec, lig, p, g, wl.dofs)      # kinds swapped
    assert e.value.code == 2
    bad = pkg.Protein(xyz=wl.lig.xyz, type=wl.lig.type + 40, mapped=wl.lig.mapped,
                      charge=wl.lig.charge)
    badid = ctx.upload_protein(bad)
    with pytest.raises(GbaError) as e:
        ctx.energy_6d(rec, badid, g, p, wl.dofs)
    assert e.value.code == 1
    ctx.release(badid)
    with pytest.raises(GbaError):
        ctx.release(badid)


def test_fp64_error_statement(small_case, oracle, ctx):
    """Error of the GPU FP32 result against the FP64 oracle, stated per pose."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    got = ctx.energy_6d(*ids, wl.dofs)
    _, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    ref64 = oracle.energy_6d_f64(wl.rec, wl.lig, grid, wl.params, wl.dofs)
    eE, eF, eT = pose_errors(got, ref64, st)
    print(f"FP32 GPU vs FP64 oracle: E max {eE.max():.2e} median {np.median(eE):.2e}; "
          f"F max {eF.max():.2e}; torque max {eT.max():.2e}")
    assert float(eE.max()) < 1e-3


@pytest.mark.parametrize("flags", [0, 1, 2, 4, 7, 8, 15])
def test_kernel_options_keep_parity(small_case, oracle, ctx, flags):
    """Each GBA_KOPT_* combination stays within the parity bound; grid and NL
    decisions are unaffected (census identical)."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    ref, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    cen0, _ = ctx.census_6d(*ids, wl.dofs)
    try:
        ctx.grid_octets(ids[2], bool(flags & 2))
        ctx.set_kernel_options(flags)
        got = ctx.energy_6d(*ids, wl.dofs)
        cen, _ = ctx.census_6d(*ids, wl.dofs)
        s, r, n = ctx.minimize_6d(*ids, wl.dofs[:16], max_evals=20)
        assert np.array_equal(ctx.energy_6d(*ids, s), r)
    finally:
        ctx.set_kernel_options(15)       # GBA_KOPT_DEFAULT
        ctx.grid_octets(ids[2], False)
    for e in pose_errors(got, ref, st):
        assert float(e.max()) <= RTOL
    assert np.array_equal(cen, cen0)


def test_force_lim_clamp_matches_oracle(small_case, oracle, ctx):
    """Deep clashes (translations scaled to 30 %) push the force sum past
    |F|^2 = 1e18, where reducePotForce scales it by 0.01 up to three times
    (src/model/reduction.h:62-72).  The oracle counts the clamps: poses
    clamped once, twice and three times occur, and the GPU results equal the
    oracle's within the parity bound on all of them (an unclamped force would
    be 100x off)."""
    wl, grid = small_case
    dofs = wl.dofs.copy()
    dofs[:, :3] *= 0.3
    with oracle.exact_sincos():
        ref, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, dofs, stats=True)
    counts = np.bincount(st["n_force_lim"], minlength=4)
    assert counts[1] > 0 and counts[2] > 0 and counts[3] > 0, counts
    got = ctx.energy_6d(*upload(ctx, wl.rec, wl.lig, grid, wl.params), dofs)
    assert np.isfinite(got).all()
    for e in pose_errors(got, ref, st):
        assert float(e.max()) <= RTOL
    clamped = st["n_force_lim"] > 0
    F = np.linalg.norm(got[clamped, 1:4].astype(np.float64), axis=1)
    assert np.all((F ** 2 <= 1.0e18 * 1.0001) | (st["n_force_lim"][clamped] == 3))
