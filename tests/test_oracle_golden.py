"""Pins the CPU oracle against the reference's own outputs.

The golden fixtures hold outputs of the reference's CPUEnergyService6D<float> /
CPUEnergyService6DModes<float> (tests/golden/make_golden.py).  On the host they
were made on the restatement is bit-identical; elsewhere libm's sinf/cosf may
differ in the last bit, hence the 1e-5 scaled bound next to the bitwise count."""
import numpy as np
import pytest

from conftest import golden_inputs, rel_err

RIGID = ["rigid_synth", "rigid_const", "rigid_pdb"]


@pytest.mark.parametrize("name", RIGID)
def test_rigid_oracle_matches_reference_fixture(name, golden_cases, oracle):
    d = golden_cases[name]
    rec, lig, params, opts = golden_inputs(d)
    grid = oracle.build_grid(rec, params, opts)
    got, st = oracle.energy_6d(rec, lig, grid, params, d["dofs"], stats=True)
    ref = d["ref_out"]
    floor = np.stack([0.05 * st["abs_E"]] + [0.05 * st["abs_F"]] * 3 + [0.05 * st["abs_T"]] * 3,
                     axis=1) + 1e-30
    assert np.all(np.isfinite(got))
    assert float(np.max(rel_err(got, ref, floor))) <= 1e-5
    # the interaction is non-trivial: NL pairs and grid beads on every pose
    assert st["n_grid"].min() > 0 and st["n_pairs"].sum() > 0


@pytest.mark.parametrize("name", RIGID)
def test_exact_sincos_oracle_bitwise_on_exact_poses(name, golden_cases, oracle):
    """With correctly rounded sin/cos the restatement equals the reference's
    outputs bit for bit on every pose whose angles the generating host's
    sinf/cosf rounded correctly -- on any host, since it no longer depends on
    the local libm."""
    d = golden_cases[name]
    rec, lig, params, opts = golden_inputs(d)
    grid = oracle.build_grid(rec, params, opts)
    with oracle.exact_sincos():
        got = oracle.energy_6d(rec, lig, grid, params, d["dofs"])
    exact = d["sincos_exact"].astype(bool)
    assert exact.mean() > 0.9
    assert np.array_equal(got[exact], d["ref_out"][exact])


def test_exact_sincos_modes_oracle_bitwise_on_exact_poses(golden_cases, oracle):
    """The modes path takes sin/cos of each angle and of its negation: where
    the generating host's libm rounded all of them correctly, the
    correctly-rounded oracle equals the reference's modes outputs bit for bit."""
    d = golden_cases["modes_synth"]
    rec, lig, params, opts = golden_inputs(d)
    gr, gl = oracle.build_grid(rec, params, opts), oracle.build_grid(lig, params, opts)
    with oracle.exact_sincos():
        got = oracle.energy_6d_modes(rec, lig, gr, gl, params, d["dofs"])
    exact = d["sincos_exact"].astype(bool)
    assert exact.mean() > 0.85
    assert np.array_equal(got[exact], d["ref_out"][exact])


def test_modes_oracle_matches_reference_fixture(golden_cases, oracle):
    d = golden_cases["modes_synth"]
    rec, lig, params, opts = golden_inputs(d)
    grid_rec = oracle.build_grid(rec, params, opts)
    grid_lig = oracle.build_grid(lig, params, opts)
    got = oracle.energy_6d_modes(rec, lig, grid_rec, grid_lig, params, d["dofs"])
    ref = d["ref_out"]
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max(axis=0, keepdims=True) + 1e-20)
    assert float(np.max(np.abs(got - ref) / scale)) <= 1e-5


def test_oracle_bitwise_equals_reference_build(small_case, oracle):
    """Where the reference compiled here (oracle/_ref), the restatement is bit-identical."""
    if not oracle.ref_available():
        pytest.skip("reference CPU path not built on this host")
    wl, grid = small_case
    a = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs)
    b = oracle.ref_energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, nworkers=3, item_size=7)
    assert np.array_equal(a, b)


def test_oracle_modes_bitwise_equals_reference_build(pkg, oracle):
    if not oracle.ref_available():
        pytest.skip("reference CPU path not built on this host")
    wl = pkg.synth.make_pair(2, 90, 70, 24, (15.0, 22.0), n_modes=4, seed=77)
    opts = pkg.GridOptions()
    gr, gl = oracle.build_grid(wl.rec, wl.params, opts), oracle.build_grid(wl.lig, wl.params, opts)
    a = oracle.energy_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, wl.dofs)
    b = oracle.ref_energy_6d_modes(wl.rec, wl.lig, gr, gl, wl.params, wl.dofs, item_size=5)
    assert np.array_equal(a, b)


def test_fp64_oracle_close_to_fp32(small_case, oracle):
    wl, grid = small_case
    a, st = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, stats=True)
    b = oracle.energy_6d_f64(wl.rec, wl.lig, grid, wl.params, wl.dofs)
    err = np.abs(a[:, 0] - b[:, 0]) / np.maximum(np.abs(b[:, 0]), 0.05 * st["abs_E"])
    assert float(err.max()) < 1e-4


def test_grid_builder_layout_and_lists(small_case, pkg):
    wl, grid = small_case
    o = pkg.GridOptions()
    assert grid.inner.numGrids == 33 and grid.outer.numGrids == 33
    assert abs(grid.outer.gridSpacing - 2 * grid.inner.gridSpacing) < 1e-7
    # NL descriptors tile the list contiguously in voxel order
    g = grid.nl_grid.reshape(-1, 2).astype(np.int64)
    assert np.all(g[1:, 1] == g[:-1, 1] + g[:-1, 0])
    assert g[-1, 1] + g[-1, 0] == grid.nl_list.shape[0]
    # brute-force one voxel's list
    v = int(np.argmax(g[:, 0]))
    Nx, Ny = grid.nl.dimN[0], grid.nl.dimN[1]
    x, y, z = v % Nx, (v // Nx) % Ny, v // (Nx * Ny)
    p = np.array(grid.nl.posMin, np.float64) + np.array([x, y, z]) * np.float64(np.float32(o.spacing))
    d2 = np.sum((wl.rec.xyz.T.astype(np.float64) - p) ** 2, axis=1)
    want = np.nonzero((d2 <= np.float64(np.float32(o.nl_cutoff)) ** 2) & (wl.rec.type > 0))[0]
    got = grid.nl_list[g[v, 1]:g[v, 1] + g[v, 0]]
    assert np.array_equal(got, want)
