"""Seeded synthetic docking workloads (there is no network for real datasets).

Each workload follows the distributions of the benchmark configurations:
  * globules: beads placed by random sequential addition, uniform in a sphere,
    rejecting candidates closer than 3.0 A to an accepted bead; radii
    20*(n/500)^(1/3) A for receptors and 15*(n/200)^(1/3) A for ligands;
    coordinates pivotized on the centroid (auto pivot, src/model/Protein.tpp:145-157);
  * types uniform in 1..32 (raw == mapped, 32 grid type channels + the charge
    channel), charges 0 / +1 / -1 with probability 0.8 / 0.1 / 0.1;
  * a symmetric 32x32 8-6 table, r0 ~ U[3,5] A, eps ~ U[0.1,10], ipon = 1,
    variable dielectric with epsilon 15 (ffelec = 332.053986/15);
  * poses: uniform random rotation (unit quaternion) turned into the
    reference's Euler angles by rotmat2euler (src/model/matrixFunctions.h:131-168),
    ligand centre uniform on a spherical shell around the receptor centre;
  * normal modes: smooth sin/cos fields of the bead coordinates with
    |k| <= 2*pi/(2R), Gram-Schmidt orthonormalised over the 3N vector,
    mode force constant 1.0, amplitudes U[-1, 1].
The random stream is numpy's PCG64 seeded with 0xA77AC7 + config id.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .model import (DIELEC_VARIABLE, FELEC, POTSHAPE_8_6, ParamTable, Protein,
                    attract_params, dofs_modes)

SEED_BASE = 0xA77AC7


def globule(rng: np.random.Generator, n: int, radius: float, min_dist: float = 3.0) -> np.ndarray:
    """(n, 3) float64 bead centres, random sequential addition in a sphere."""
    pts = np.empty((n, 3), dtype=np.float64)
    k = 0
    md2 = min_dist * min_dist
    tries = 0
    batch = 64
    while k < n:
        cand = rng.normal(size=(batch, 3))
        cand /= np.linalg.norm(cand, axis=1, keepdims=True)
        cand *= radius * rng.random((batch, 1)) ** (1.0 / 3.0)
        for c in cand:
            tries += 1
            if k == 0 or np.min(np.sum((pts[:k] - c) ** 2, axis=1)) >= md2:
                pts[k] = c
                k += 1
                if k == n:
                    break
        if tries > 1000 * n:
            raise RuntimeError(f"globule: cannot place {n} beads in radius {radius}")
    return pts


def receptor_radius(n: int) -> float:
    return 20.0 * (n / 500.0) ** (1.0 / 3.0)


def ligand_radius(n: int) -> float:
    return 15.0 * (n / 200.0) ** (1.0 / 3.0)


def make_protein(rng: np.random.Generator, n: int, radius: float, n_types: int = 32,
                 n_modes: int = 0) -> Protein:
    pts = globule(rng, n, radius)
    xyz = pts.T.astype(np.float32)
    xyz = (xyz - xyz.mean(axis=1, keepdims=True)).astype(np.float32)
    types = rng.integers(1, n_types + 1, size=n).astype(np.uint32)
    charge = rng.choice(np.array([0.0, 1.0, -1.0], dtype=np.float32), size=n, p=[0.8, 0.1, 0.1])
    modes = mode_force = None
    if n_modes:
        modes = make_modes(rng, xyz, n_modes, radius)
        mode_force = np.ones(n_modes, dtype=np.float32)
    return Protein(xyz=xyz, type=types, mapped=types.copy(), charge=charge.astype(np.float32),
                   modes=modes, mode_force=mode_force)


def make_modes(rng: np.random.Generator, xyz: np.ndarray, n_modes: int, radius: float) -> np.ndarray:
    """(3, n, M) orthonormal smooth displacement fields."""
    n = xyz.shape[1]
    X = xyz.T.astype(np.float64)
    kmax = 2.0 * np.pi / (2.0 * radius)
    vecs = []
    while len(vecs) < n_modes:
        field = np.empty((n, 3))
        for a in range(3):
            k = rng.normal(size=3)
            k *= kmax * rng.random() / np.linalg.norm(k)
            phase = rng.uniform(0, 2 * np.pi)
            f = np.sin if rng.random() < 0.5 else np.cos
            field[:, a] = f(X @ k + phase)
        v = field.T.ravel()            # 3N vector, axis-major
        for u in vecs:
            v = v - np.dot(u, v) * u
        nv = np.linalg.norm(v)
        if nv > 1e-6:
            vecs.append(v / nv)
    M = np.stack(vecs, axis=0).reshape(n_modes, 3, n)   # [m][axis][i]
    return np.ascontiguousarray(M.transpose(1, 2, 0)).astype(np.float32)   # (3, n, M)


def make_params(rng: np.random.Generator, n_types: int = 32, epsilon: float = 15.0) -> ParamTable:
    r0 = rng.uniform(3.0, 5.0, size=(n_types, n_types))
    eps = rng.uniform(0.1, 10.0, size=(n_types, n_types))
    r0 = np.triu(r0) + np.triu(r0, 1).T
    eps = np.triu(eps) + np.triu(eps, 1).T
    table = attract_params(r0.astype(np.float32), eps.astype(np.float32), potshape=POTSHAPE_8_6)
    return ParamTable(table=table, potshape=POTSHAPE_8_6, dielec=DIELEC_VARIABLE,
                      ffelec=float(np.float32(FELEC / epsilon)))


def rotmat2euler(m: np.ndarray) -> np.ndarray:
    """rotmat2euler, src/model/matrixFunctions.h:131-168, for (n, 9) row-major matrices.

    The gimbal-lock branch keeps the reference's test `abs(rotmat[8] >= 0.9999)`,
    i.e. it triggers on rotmat[8] >= 0.9999 only."""
    phi = np.arctan2(m[:, 5], m[:, 2])
    ssi = np.arccos(np.clip(m[:, 8], -1.0, 1.0))
    rot = np.arctan2(-m[:, 7], -m[:, 6])
    lock = m[:, 8] >= 0.9999
    if np.any(lock):
        for i in np.nonzero(lock)[0]:
            r = m[i]
            p = 0.0
            if abs(r[0]) >= 0.9999:
                ro = np.pi if r[0] < 0.0 else 0.0
                s = np.pi if r[8] < 0.0 else 0.0
            else:
                if r[8] < 0.0:
                    s = np.pi
                    ro = -np.arccos(-r[0])
                else:
                    s = 0.0
                    ro = np.arccos(r[0])
            if r[1] < 0:
                ro *= -1.0
            phi[i], ssi[i], rot[i] = p, s, ro
    return np.stack([phi, ssi, rot], axis=1)


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """(n, 9) uniformly distributed rotation matrices (random unit quaternions)."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
        2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
        2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], axis=1)


def random_poses(rng: np.random.Generator, n: int, r_min: float, r_max: float) -> np.ndarray:
    """(n, 6) float32 DOF_6D records {pos xyz, ang xyz}: centre on a shell."""
    ang = rotmat2euler(random_rotations(rng, n))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = (r_min ** 3 + rng.random(n) * (r_max ** 3 - r_min ** 3)) ** (1.0 / 3.0)
    pos = d * r[:, None]
    return np.concatenate([pos, ang], axis=1).astype(np.float32)


@dataclass
class Workload:
    """One receptor-ligand pair with its poses (grids are built separately)."""
    name: str
    rec: Protein
    lig: Protein
    params: ParamTable
    dofs: np.ndarray                  # (n, 6) or (n, 26) for modes
    steps: int = 0                    # minimizer evaluation budget
    modes: bool = False


# Shells as the workload descriptions state them (configs 0, 1, 3).  Config 2
# states none: its globules (radii 28.8 and 21.6 A) touch at about 50 A, so
# its centres lie on a 45-55 A shell, around contact.
CONFIGS = {
    0: dict(rec=500, lig=200, poses=1000, shell=(35.0, 45.0), steps=100),
    1: dict(rec=2000, lig=700, poses=100_000, shell=(40.0, 55.0), steps=0),
    2: dict(rec=1500, lig=600, poses=50_000, shell=(45.0, 55.0), steps=200, modes=5),
    3: dict(rec=2000, lig=700, poses=10_000, shell=(40.0, 55.0), steps=0),
}


def make_pair(config_id: int, n_rec: int, n_lig: int, n_poses: int, shell, steps: int = 0,
              n_modes: int = 0, seed: int | None = None, name: str | None = None) -> Workload:
    rng = np.random.default_rng(SEED_BASE + config_id if seed is None else seed)
    params = make_params(rng)
    rec = make_protein(rng, n_rec, receptor_radius(n_rec), n_modes=n_modes)
    lig = make_protein(rng, n_lig, ligand_radius(n_lig), n_modes=n_modes)
    dofs = random_poses(rng, n_poses, *shell)
    if n_modes:
        amps_r = rng.uniform(-1, 1, size=(n_poses, n_modes)).astype(np.float32)
        amps_l = rng.uniform(-1, 1, size=(n_poses, n_modes)).astype(np.float32)
        dofs = dofs_modes(dofs, amps_r, amps_l)
    return Workload(name=name or f"config{config_id}", rec=rec, lig=lig, params=params,
                    dofs=dofs, steps=steps, modes=bool(n_modes))


def make_config(config_id: int, n_poses: int | None = None) -> Workload:
    """The synthetic workload of benchmark configuration 0..3 (4: make_batch)."""
    c = CONFIGS[config_id]
    return make_pair(config_id, c["rec"], c["lig"], n_poses or c["poses"], c["shell"],
                     steps=c.get("steps", 0), n_modes=c.get("modes", 0))


def make_batch(n_pairs: int = 64, seed: int = SEED_BASE + 4, pose_scale: float = 1.0,
               rec_range=(300, 3000), lig_range=(100, 1500), pose_range=(2000, 50000)) -> list:
    """Configuration 4: pairs of uneven sizes, each with its own table draw."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_pairs):
        nr = int(rng.integers(rec_range[0], rec_range[1] + 1))
        nl = int(rng.integers(lig_range[0], lig_range[1] + 1))
        npz = max(1, int(int(rng.integers(pose_range[0], pose_range[1] + 1)) * pose_scale))
        out.append(make_pair(4, nr, nl, npz, (35.0, 45.0), steps=500,
                             seed=int(rng.integers(0, 2**63 - 1)), name=f"pair{k:02d}"))
    return out
