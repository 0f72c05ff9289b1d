"""Writes the golden fixtures in tests/golden/ from the reference's OWN CPU path.

Run in a tree where the reference sources were compiled into
oracle/_ref/libattract_ref.so (oracle/build_ref.sh).  Each fixture stores the
inputs (pivotized beads, types, charges, modes, the parameter table, grid
options, poses) and the reference's outputs for them, computed through its
Server<Types_6D<float>> + CPUEnergyService6D<float> (or the modes variant);
rigid fixtures also mark the poses whose sin/cos the generating host's libm
rounded correctly (sincos_exact).
Grids are not stored: tests rebuild them with the oracle's CPU grid builder,
which is deterministic, and feed the identical grid to every path.

Fixtures:
  rigid_synth   synthetic pair (config-0 distributions, 150/60 beads), 96 poses
  rigid_pdb     the reference's own test proteins test/resources/receptorr.pdb and
                ligandr.pdb with test/resources/attract.par (types 1..31), 64 poses
  rigid_const   synthetic pair, constant dielectric, fractional charges, 48 poses
  modes_synth   synthetic pair with 3 modes each side, receptor and ligand grids, 48 poses
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

pkg = __graft_entry__.load_package()
from oracle import pyoracle as po  # noqa: E402

REF_TEST = po.ref_root() / "test" / "resources"
OUT = Path(__file__).resolve().parent


def sincos_mask(dofs):
    """Per rigid pose: whether this host's sinf/cosf (the ones the reference
    called) returned the correctly rounded value for all three angles -- the
    poses on which a device summing in the reference's order must equal
    ref_out bit for bit."""
    return po.libm_sincos_rounds_exactly(np.asarray(dofs)[:, 3:6])


def pack(name, rec, lig, params, opts, dofs, out, extra=None):
    tab = np.stack([params.table[k].astype(np.float64) for k in ("rc", "ac", "ipon", "rmin2", "emin")],
                   axis=1).astype(np.float32)
    d = dict(rec_xyz=rec.xyz, rec_type=rec.type, rec_mapped=rec.mapped, rec_charge=rec.charge,
             lig_xyz=lig.xyz, lig_type=lig.type, lig_mapped=lig.mapped, lig_charge=lig.charge,
             table=tab, potshape=np.int32(params.potshape), dielec=np.int32(params.dielec),
             ffelec=np.float32(params.ffelec), alphabet=np.asarray(opts.alphabet, np.uint32),
             dofs=dofs, ref_out=out)
    for p, prefix in ((rec, "rec"), (lig, "lig")):
        if p.n_modes:
            d[prefix + "_modes"] = p.modes
            d[prefix + "_mode_force"] = p.mode_force
    if extra:
        d.update(extra)
    np.savez_compressed(OUT / f"{name}.npz", **d)
    print(f"wrote {name}.npz: {dofs.shape[0]} poses")


def auto_pivot(xyz):
    """Protein::auto_pivotize (src/model/Protein.tpp:145-157): float sums, /n."""
    piv = np.array([np.cumsum(xyz[a], dtype=np.float32)[-1] for a in range(3)], np.float32)
    piv = (piv / np.float32(xyz.shape[1])).astype(np.float32)
    return (xyz - piv[:, None]).astype(np.float32)


def rigid_synth():
    wl = pkg.synth.make_pair(0, 150, 60, 96, (18.0, 27.0), seed=101)
    opts = pkg.GridOptions()
    grid = po.build_grid(wl.rec, wl.params, opts)
    out = po.ref_energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, nworkers=2, item_size=17)
    pack("rigid_synth", wl.rec, wl.lig, wl.params, opts, wl.dofs, out, dict(sincos_exact=sincos_mask(wl.dofs)))


def rigid_const():
    wl = pkg.synth.make_pair(0, 120, 50, 48, (16.0, 23.0), seed=202)
    for p in (wl.rec, wl.lig):
        p.charge[:] = np.where(p.charge != 0, np.float32(0.35) * np.sign(p.charge), 0).astype(np.float32)
    wl.params.dielec = pkg.DIELEC_CONSTANT
    opts = pkg.GridOptions()
    grid = po.build_grid(wl.rec, wl.params, opts)
    out = po.ref_energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs, nworkers=1, item_size=100)
    pack("rigid_const", wl.rec, wl.lig, wl.params, opts, wl.dofs, out, dict(sincos_exact=sincos_mask(wl.dofs)))


def rigid_pdb():
    rxyz, rtype, rq = po.ref_read_pdb(str(REF_TEST / "receptorr.pdb"), default_map=True)
    lxyz, ltype, lq = po.ref_read_pdb(str(REF_TEST / "ligandr.pdb"), default_map=True)
    table, potshape = po.ref_read_params(str(REF_TEST / "attract.par"))
    T = int(round(np.sqrt(table.shape[0])))
    keep = 31   # receptorgrid.alphabet lists types 1..31 (+99 -> 0)
    table = table.reshape(T, T)[:keep, :keep].ravel().copy()
    alphabet = list(range(1, keep + 1))
    rec = pkg.Protein(xyz=auto_pivot(rxyz), type=rtype, mapped=rtype.copy(), charge=rq)
    # ligand mapped types through the alphabet (createTypeMapFromVector, src/model/TypeMap.h:57-66)
    lig = pkg.Protein(xyz=auto_pivot(lxyz), type=ltype, mapped=ltype.copy(), charge=lq)
    params = pkg.ParamTable(table=table, potshape=potshape, dielec=pkg.DIELEC_VARIABLE,
                            ffelec=float(np.float32(pkg.FELEC / 15.0)))
    opts = pkg.GridOptions(alphabet=alphabet)
    grid = po.build_grid(rec, params, opts)
    rng = np.random.default_rng(303)
    dofs = pkg.synth.random_poses(rng, 64, 22.0, 32.0)
    out = po.ref_energy_6d(rec, lig, grid, params, dofs, nworkers=2, item_size=100)
    pack("rigid_pdb", rec, lig, params, opts, dofs, out, dict(sincos_exact=sincos_mask(dofs)))


def modes_synth():
    wl = pkg.synth.make_pair(2, 110, 60, 48, (17.0, 24.0), n_modes=3, seed=404)
    opts = pkg.GridOptions()
    grid_rec = po.build_grid(wl.rec, wl.params, opts)
    grid_lig = po.build_grid(wl.lig, wl.params, opts)
    out = po.ref_energy_6d_modes(wl.rec, wl.lig, grid_rec, grid_lig, wl.params, wl.dofs,
                                 nworkers=2, item_size=10)
    # the modes path takes sin/cos of the angles and of their negations (invertDOF)
    ang = np.ascontiguousarray(wl.dofs[:, 3:6])
    exact = sincos_mask(wl.dofs) & po.libm_sincos_rounds_exactly(-ang)
    pack("modes_synth", wl.rec, wl.lig, wl.params, opts, wl.dofs, out, dict(sincos_exact=exact))


if __name__ == "__main__":
    if not po.ref_available():
        sys.exit("oracle/_ref/libattract_ref.so missing: run oracle/build_ref.sh first")
    rigid_synth()
    rigid_const()
    rigid_pdb()
    modes_synth()
