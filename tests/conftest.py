"""Shared fixtures.  `gpu`-marked tests need a CUDA device and the built
library; everything else runs on the CPU (oracle, host logic, C-ABI loading)."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

PKG = __graft_entry__.load_package()
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and libgbattract")


@pytest.fixture(scope="session")
def pkg():
    return PKG


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    if not pyoracle.ORACLE_LIB.exists():
        import subprocess
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    return pyoracle


def _small_pair(seed: int, n_rec: int = 150, n_lig: int = 60, n_poses: int = 128,
                shell=(18.0, 26.0)):
    return PKG.synth.make_pair(0, n_rec, n_lig, n_poses, shell, seed=seed)


@pytest.fixture(scope="session")
def small_case(oracle):
    """A small receptor-ligand pair with contact poses and its CPU-built grid."""
    wl = _small_pair(11)
    grid = oracle.build_grid(wl.rec, wl.params, PKG.GridOptions())
    return wl, grid


@pytest.fixture(scope="session")
def golden_cases():
    """Committed golden fixtures written by tests/golden/make_golden.py."""
    out = {}
    for f in sorted(GOLDEN.glob("*.npz")):
        out[f.stem] = dict(np.load(f, allow_pickle=False))
    return out


def golden_inputs(d: dict):
    """Rebuilds Protein / ParamTable objects from a golden npz dict."""
    m = PKG.model

    def prot(prefix):
        modes = d.get(prefix + "_modes")
        mf = d.get(prefix + "_mode_force")
        return m.Protein(xyz=d[prefix + "_xyz"], type=d[prefix + "_type"],
                         mapped=d[prefix + "_mapped"], charge=d[prefix + "_charge"],
                         modes=modes if modes is not None and modes.size else None,
                         mode_force=mf if mf is not None and mf.size else None)

    table = np.zeros(d["table"].shape[0], m.FFPARAM_DTYPE)
    for k, name in enumerate(("rc", "ac", "ipon", "rmin2", "emin")):
        table[name] = d["table"][:, k].astype(table.dtype[name])
    params = m.ParamTable(table=table, potshape=int(d["potshape"]), dielec=int(d["dielec"]),
                          ffelec=float(d["ffelec"]))
    opts = m.GridOptions(alphabet=[int(a) for a in d["alphabet"]])
    return prot("rec"), prot("lig"), params, opts


def rel_err(got: np.ndarray, ref: np.ndarray, floor: np.ndarray) -> np.ndarray:
    """|got - ref| / max(|ref|, floor), elementwise."""
    return np.abs(got.astype(np.float64) - ref.astype(np.float64)) / np.maximum(
        np.abs(ref.astype(np.float64)), floor)
