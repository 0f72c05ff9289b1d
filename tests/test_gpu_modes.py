"""Parity of the fused normal-mode kernel with the reference CPU modes path
(golden fixture of CPUEnergyService6DModes<float>) and with the oracle.

Tolerance per pose: energy, force and torque as in test_gpu_rigid (1e-4 of
max(|ref|, 0.05 S)); mode-gradient vectors within 1e-4 of
max(|ref|, 1e-3 * max over the batch) -- they are sums over every bead of both
proteins and pass through the delta + 4 k delta^4 correction."""
import numpy as np
import pytest

from conftest import golden_inputs
from test_gpu_rigid import pose_errors, upload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(pkg):
    from gbattract.context import GbaContext
    c = GbaContext(0)
    yield c
    c.close()


def mode_errors(got, ref, Mr, Ml):
    errs = []
    for lo, M in ((7, Mr), (17, Ml)):
        g = got[:, lo:lo + M].astype(np.float64)
        r = ref[:, lo:lo + M].astype(np.float64)
        fin = np.all(np.isfinite(r), axis=1)
        assert np.array_equal(np.isfinite(g).all(axis=1), fin)
        g, r = g[fin], r[fin]
        if len(r) == 0:
            continue
        nr = np.linalg.norm(r, axis=1)
        floor = 1e-3 * nr.max() + 1e-30
        errs.append(np.linalg.norm(g - r, axis=1) / np.maximum(nr, floor))
    return np.concatenate(errs) if errs else np.zeros(1)


def run_modes(ctx, oracle, rec, lig, params, opts, dofs, octets=False):
    gr = oracle.build_grid(rec, params, opts)
    gl = oracle.build_grid(lig, params, opts)
    ids = (ctx.upload_protein(rec), ctx.upload_protein(lig), ctx.upload_grid(gr),
           ctx.upload_grid(gl), ctx.upload_params(params))
    if octets:               # cooperative 8-lane lookups in both passes
        ctx.grid_octets(ids[2], True)
        ctx.grid_octets(ids[3], True)
    return ctx.energy_6d_modes(*ids, dofs), gr, gl


def test_golden_modes_reference_outputs(golden_cases, oracle, ctx):
    d = golden_cases["modes_synth"]
    rec, lig, params, opts = golden_inputs(d)
    got, gr, gl = run_modes(ctx, oracle, rec, lig, params, opts, d["dofs"])
    ref = d["ref_out"]
    _, st = oracle.energy_6d_modes(rec, lig, gr, gl, params, d["dofs"], stats=True)
    for e in pose_errors(got[:, :7], ref[:, :7], st):
        assert float(e.max()) <= 1e-4
    assert float(mode_errors(got, ref, rec.n_modes, lig.n_modes).max()) <= 1e-4
    # unused mode slots stay zero
    assert np.all(got[:, 7 + rec.n_modes:17] == 0) and np.all(got[:, 17 + lig.n_modes:] == 0)


@pytest.mark.parametrize("octets", [False, True])
def test_modes_fresh_case_vs_oracle(pkg, oracle, ctx, octets):
    wl = pkg.synth.make_pair(2, 130, 70, 96, (16.0, 24.0), n_modes=5, seed=515)
    opts = pkg.GridOptions()
    got, gr, gl = run_modes(ctx, oracle, wl.rec, wl.lig, wl.params, opts, wl.dofs, octets)
    ref, st = oracle.energy_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, wl.dofs, stats=True)
    for e in pose_errors(got[:, :7], ref[:, :7], st):
        assert float(e.max()) <= 1e-4
    assert float(mode_errors(got, ref, 5, 5).max()) <= 1e-4


@pytest.mark.parametrize("n_modes", [8, 10])
def test_more_than_five_modes(pkg, oracle, ctx, n_modes):
    """Mode counts above five run the kernels compiled for the full capacity
    of ten (MODES_MAX, src/model/Types_6D_Config.h:11): scoring against the
    oracle, and the device minimizer equal to the plain per-step form."""
    wl = pkg.synth.make_pair(2, 120, 60, 64, (16.0, 24.0), n_modes=n_modes, seed=818 + n_modes)
    opts = pkg.GridOptions()
    got, gr, gl = run_modes(ctx, oracle, wl.rec, wl.lig, wl.params, opts, wl.dofs, octets=True)
    ref, st = oracle.energy_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, wl.dofs, stats=True)
    fin = np.isfinite(ref).all(axis=1)
    assert fin.mean() > 0.9
    for e in pose_errors(got[fin, :7], ref[fin, :7], st[fin]):
        assert float(e.max()) <= 1e-4
    assert float(mode_errors(got[fin], ref[fin], n_modes, n_modes).max()) <= 1e-4
    ids = (ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_grid(gr), ctx.upload_grid(gl),
           ctx.upload_params(wl.params))
    s1, r1, n1 = ctx.minimize_6d_modes(*ids, wl.dofs[:32], max_evals=40)
    s2, r2, n2 = ctx.minimize_6d_modes_plain(*ids, wl.dofs[:32], max_evals=40)
    assert np.array_equal(n1, n2)
    assert np.array_equal(r1, r2, equal_nan=True) and np.array_equal(s1, s2, equal_nan=True)
    for i in ids:
        ctx.release(i)


def test_modes_minimizer_device_plain_and_oracle(pkg, oracle, ctx):
    """Device VA13 over 6 + Mr + Ml DOF == the plain per-step form bit for bit;
    against the CPU oracle's VA13 neither side ends lower more often and the
    median minimized energies agree."""
    wl = pkg.synth.make_pair(2, 120, 60, 128, (18.0, 27.0), n_modes=3, seed=717)
    opts = pkg.GridOptions()
    gr, gl = oracle.build_grid(wl.rec, wl.params, opts), oracle.build_grid(wl.lig, wl.params, opts)
    ids = (ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_grid(gr),
           ctx.upload_grid(gl), ctx.upload_params(wl.params))
    s1, r1, n1 = ctx.minimize_6d_modes(*ids, wl.dofs, max_evals=60)
    s2, r2, n2 = ctx.minimize_6d_modes_plain(*ids, wl.dofs, max_evals=60)
    # a pose in a deep clash can overflow correctModeForce's 4 k delta^4 to
    # inf and end in NaN -- identically in both forms
    assert np.array_equal(n1, n2)
    assert np.array_equal(s1, s2, equal_nan=True) and np.array_equal(r1, r2, equal_nan=True)
    assert n1.max() <= 61
    s3, r3i, n3 = ctx.minimize_6d_modes_plain(*ids, wl.dofs, max_evals=60, item_size=100)
    assert np.array_equal(n1, n3)
    assert np.array_equal(s1, s3, equal_nan=True) and np.array_equal(r1, r3i, equal_nan=True)
    fin = np.isfinite(s1).all(axis=1) & np.isfinite(r1).all(axis=1)
    assert fin.mean() >= 0.9
    assert np.array_equal(ctx.energy_6d_modes(*ids, s1[fin]), r1[fin])
    # the minimizer descends (mode entries are gradients, position and angle
    # entries forces)
    e0 = ctx.energy_6d_modes(*ids, wl.dofs)[:, 0]
    assert np.mean(r1[fin, 0] <= e0[fin]) >= 0.9
    _, r3, _ = oracle.minimize_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, wl.dofs, 60)
    d1 = wl.dofs.copy()
    d1[:, 0] = np.nextafter(d1[:, 0], np.float32(np.inf))
    _, r4, _ = oracle.minimize_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, d1, 60)
    st = oracle.minimization_stats(r1, r3)
    print(f"modes minimization, device vs oracle: {st}; oracle with a one-ulp start perturbation "
          f"within 1e-3: {oracle.minimization_stats(r4, r3)['within_tol']:.3f}")
    # symmetric: neither side ends lower more often, the distributions agree
    assert abs(st["a_at_least_as_low"] - st["b_at_least_as_low"]) <= 0.1
    assert abs(st["a_quantiles"][2] - st["b_quantiles"][2]) <= 0.05 * abs(st["b_quantiles"][2]) + 0.5
    # octet grids (cooperative lookups): device and plain forms still agree bit for bit
    ctx.grid_octets(ids[2], True)
    ctx.grid_octets(ids[3], True)
    s5, r5, n5 = ctx.minimize_6d_modes(*ids, wl.dofs[:32], max_evals=30)
    s6, r6, n6 = ctx.minimize_6d_modes_plain(*ids, wl.dofs[:32], max_evals=30)
    assert np.array_equal(n5, n6)
    assert np.array_equal(s5, s6, equal_nan=True) and np.array_equal(r5, r6, equal_nan=True)


def test_zero_amplitudes_match_rigid(small_case, pkg, oracle, ctx):
    """With no modes the flexible kernel reduces to the rigid one (ligand side)."""
    wl, grid = small_case
    ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
    rigid = ctx.energy_6d(*ids, wl.dofs)
    gl = oracle.build_grid(wl.lig, wl.params, pkg.GridOptions())
    glid = ctx.upload_grid(gl)
    d26 = pkg.dofs_modes(wl.dofs)
    got = ctx.energy_6d_modes(ids[0], ids[1], ids[2], glid, ids[3], d26)
    # same terms, summed in a different order by the two kernels
    _, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    for e in pose_errors(got[:, :7], rigid, st):
        assert float(e.max()) <= 1e-5
    assert np.all(got[:, 7:] == 0)


def test_modes_pose_counter_visits_every_pose_once(pkg, oracle, ctx):
    """Warps of the modes kernel claim poses from a per-launch counter: a
    batch larger than the resident warps gives every pose its own result,
    bit for bit the same as the pose scored in small batches (NaN where the
    deformation overflows, in the same places)."""
    wl = pkg.synth.make_pair(2, 130, 70, 96, (16.0, 24.0), n_modes=5, seed=515)
    rng = np.random.default_rng(5)
    n = 5003
    dofs = wl.dofs[rng.integers(0, len(wl.dofs), n)].copy()
    dofs[:, :3] += rng.normal(0, 2.0, (n, 3)).astype(np.float32)
    gr = oracle.build_grid(wl.rec, wl.params, pkg.GridOptions())
    gl = oracle.build_grid(wl.lig, wl.params, pkg.GridOptions())
    ids = (ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_grid(gr),
           ctx.upload_grid(gl), ctx.upload_params(wl.params))
    whole = ctx.energy_6d_modes(*ids, dofs)
    pieces = np.concatenate([ctx.energy_6d_modes(*ids, dofs[k:k + 333]) for k in range(0, n, 333)])
    assert np.array_equal(whole, pieces, equal_nan=True)
