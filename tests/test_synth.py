"""The seeded synthetic workload generator."""
import numpy as np


def test_globule_spacing_and_determinism(pkg):
    rng = np.random.default_rng(1)
    p = pkg.synth.globule(rng, 300, pkg.synth.receptor_radius(300))
    d2 = np.sum((p[:, None, :] - p[None, :, :]) ** 2, axis=2)
    np.fill_diagonal(d2, np.inf)
    assert d2.min() >= 9.0 - 1e-9
    assert np.all(np.linalg.norm(p, axis=1) <= pkg.synth.receptor_radius(300) + 1e-9)
    q = pkg.synth.globule(np.random.default_rng(1), 300, pkg.synth.receptor_radius(300))
    assert np.array_equal(p, q)


def test_config_distributions(pkg):
    wl = pkg.synth.make_config(0)
    assert wl.rec.n == 500 and wl.lig.n == 200 and wl.dofs.shape == (1000, 6)
    assert wl.rec.type.min() >= 1 and wl.rec.type.max() <= 32
    frac = np.mean(wl.rec.charge != 0)
    assert 0.1 < frac < 0.3
    assert abs(float(wl.rec.xyz.mean())) < 1e-3        # pivotized
    r = np.linalg.norm(wl.dofs[:, :3], axis=1)
    assert r.min() >= 35.0 - 1e-3 and r.max() <= 45.0 + 1e-3
    assert wl.params.num_types == 32
    t = wl.params.table.reshape(32, 32)
    assert np.array_equal(t["rc"], t["rc"].T)          # symmetric table


def test_rotmat2euler_roundtrip(pkg):
    """rotmat2euler followed by the reference's euler2rotmat recovers the rotation."""
    rng = np.random.default_rng(3)
    m = pkg.synth.random_rotations(rng, 500)
    a = pkg.synth.rotmat2euler(m)
    phi, ssi, rot = a.T
    cs, cp, ss, sp, cr, sr = np.cos(ssi), np.cos(phi), np.sin(ssi), np.sin(phi), np.cos(rot), np.sin(rot)
    r = np.stack([cr * cs * cp + sr * sp, sr * cs * cp - cr * sp, ss * cp,
                  cr * cs * sp - sr * cp, sr * cs * sp + cr * cp, ss * sp,
                  -cr * ss, -sr * ss, cs], axis=1)
    assert np.max(np.abs(r - m)) < 1e-9


def test_modes_orthonormal(pkg):
    wl = pkg.synth.make_pair(2, 80, 40, 4, (30, 35), n_modes=5, seed=9)
    M = wl.rec.modes.transpose(2, 0, 1).reshape(5, -1).astype(np.float64)
    assert np.allclose(M @ M.T, np.eye(5), atol=1e-5)
    assert wl.dofs.shape == (4, 26)


def test_batch_sizes(pkg):
    pairs = pkg.synth.make_batch(n_pairs=3, pose_scale=0.01)
    for p in pairs:
        assert 300 <= p.rec.n <= 3000 and 100 <= p.lig.n <= 1500
