"""Host-side data containers of the docking energy path (numpy, no compute).

They mirror the reference's model types field for field:
  Protein     src/model/Protein.h:39-167   (SoA coordinates, types, charges, modes)
  ParamTable  src/model/ParamTable.h:18-101 + SimParam src/model/SimParam.h:39-55
  GridSet     src/model/GridUnion.h:20 (inner/outer IntrplGrid + NLGrid), in the
              memory layout readGridFromGridFile builds (src/fileIO/readFile.cpp:261-422)
Pose arrays are float32 (n, 6) = DOF_6D {pos xyz, ang xyz} and results (n, 7)
= Result_6D {E, pos xyz, ang xyz}; the normal-mode records are (n, 26) and
(n, 27) with GBA_MODES_MAX = 10 receptor then 10 ligand amplitudes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

MODES_MAX = 10           # MODES_MAX_NUMBER, src/model/Types_6D_Config.h:11
FELEC = 332.053986       # src/model/SimParam.h:31
POTSHAPE_12_6 = 0
POTSHAPE_8_6 = 1
DIELEC_CONSTANT = 0
DIELEC_VARIABLE = 1

DOF_WIDTH = 6
RESULT_WIDTH = 7
DOF_MODES_WIDTH = 6 + 2 * MODES_MAX
RESULT_MODES_WIDTH = 7 + 2 * MODES_MAX

FFPARAM_DTYPE = np.dtype([("rc", "<f4"), ("ac", "<f4"), ("ipon", "<i4"),
                          ("rmin2", "<f4"), ("emin", "<f4")])


@dataclass
class Protein:
    """A coarse-grained protein, pivotized (coordinates relative to its pivot)."""
    xyz: np.ndarray                  # (3, n) float32, SoA
    type: np.ndarray                 # (n,) uint32 raw type after the default map (0 = dummy)
    mapped: np.ndarray               # (n,) uint32 channel of the partner's grid (0 = none)
    charge: np.ndarray               # (n,) float32
    modes: np.ndarray | None = None  # (3, n, M) float32: x[i*M+m] then y then z
    mode_force: np.ndarray | None = None  # (M,) float32

    def __post_init__(self):
        self.xyz = np.ascontiguousarray(self.xyz, dtype=np.float32)
        self.type = np.ascontiguousarray(self.type, dtype=np.uint32)
        self.mapped = np.ascontiguousarray(self.mapped, dtype=np.uint32)
        self.charge = np.ascontiguousarray(self.charge, dtype=np.float32)
        if self.xyz.shape != (3, self.n):
            raise ValueError("xyz must be (3, n)")
        if self.modes is not None:
            self.modes = np.ascontiguousarray(self.modes, dtype=np.float32)
            self.mode_force = np.ascontiguousarray(self.mode_force, dtype=np.float32)
            if self.modes.shape[:2] != (3, self.n) or self.modes.shape[2] > MODES_MAX:
                raise ValueError("modes must be (3, n, M) with M <= 10")

    @property
    def n(self) -> int:
        return int(self.type.shape[0])

    @property
    def n_modes(self) -> int:
        return 0 if self.modes is None else int(self.modes.shape[2])


@dataclass
class ParamTable:
    """ATTRACT pair parameters after the attract.par transform plus SimParam."""
    table: np.ndarray                # (T*T,) FFPARAM_DTYPE, index T*typeA + typeB
    potshape: int = POTSHAPE_8_6
    dielec: int = DIELEC_VARIABLE
    ffelec: float = float(np.float32(FELEC / 15.0))

    @property
    def num_types(self) -> int:
        return int(round(np.sqrt(self.table.shape[0])))


def attract_params(r0: np.ndarray, eps: np.ndarray, ipon: np.ndarray | None = None,
                   potshape: int = POTSHAPE_8_6) -> np.ndarray:
    """The attract.par -> ParamTable transform of src/fileIO/readFile.cpp:484-512.

    r0, eps: (T, T) arrays [typeA][typeB].  Products are formed in double from
    the float32 inputs and stored as float32, as std::pow(float, unsigned) does.
    """
    r0 = np.asarray(r0, dtype=np.float32).astype(np.float64)
    eps = np.asarray(eps, dtype=np.float32).astype(np.float64)
    T = r0.shape[0]
    out = np.zeros(T * T, dtype=FFPARAM_DTYPE)
    if ipon is None:
        ipon = np.ones((T, T), dtype=np.int32)
    if potshape == POTSHAPE_8_6:
        rc = (eps * r0 ** 8).astype(np.float32)
        ac = (eps * r0 ** 6).astype(np.float32)
        rc64, ac64 = rc.astype(np.float64), ac.astype(np.float64)
        ok = (ac > 0) & (rc > 0)
        with np.errstate(divide="ignore", invalid="ignore"):
            emin = np.where(ok, -27.0 * ac64 ** 4 / (256.0 * rc64 ** 3), 0.0).astype(np.float32)
            rmin2 = np.where(ok, (np.float32(4.0) * rc) / (np.float32(3.0) * ac), 0.0).astype(np.float32)
    else:
        rc = (eps * r0 ** 12).astype(np.float32)
        ac = (eps * r0 ** 6).astype(np.float32)
        emin = (-0.25 * eps).astype(np.float32)
        rmin2 = (np.float32(1.25992105) * r0.astype(np.float32) * r0.astype(np.float32)).astype(np.float32)
    out["rc"] = rc.ravel()
    out["ac"] = ac.ravel()
    out["ipon"] = np.asarray(ipon, dtype=np.int32).ravel()
    out["rmin2"] = rmin2.ravel()
    out["emin"] = emin.ravel()
    return out


@dataclass
class IntrplDesc:
    """IntrplGrid::Desc without typemask (src/model/IntrplGrid.h:183-207)."""
    numGrids: int
    dimN: tuple
    gridSpacing: float
    posMin: tuple

    @property
    def nvox(self) -> int:
        return int(self.dimN[0]) * int(self.dimN[1]) * int(self.dimN[2])


@dataclass
class NLDesc:
    """NLGrid::Desc (src/model/NLGrid.h:151-165)."""
    dimN: tuple
    gridSpacing: float
    dPlateau: float
    posMin: tuple
    numEl: int = 0


@dataclass
class GridSet:
    """Inner + outer interpolation grids and the neighbour-list grid.

    inner_data/outer_data: (numGrids, Nz, Ny, Nx, 4) float32, channel 0 = charge.
    nl_grid: (Nz, Ny, Nx, 2) uint32 {numEl, idx}; nl_list: (numEl,) uint32.
    """
    inner: IntrplDesc
    inner_data: np.ndarray
    outer: IntrplDesc
    outer_data: np.ndarray
    nl: NLDesc
    nl_grid: np.ndarray
    nl_list: np.ndarray

    def nbytes(self) -> int:
        return int(self.inner_data.nbytes + self.outer_data.nbytes + self.nl_grid.nbytes +
                   self.nl_list.nbytes)


@dataclass
class GridOptions:
    """Grid builder settings (inner 0.9 A, outer 1.8 A, plateau 10 A, NL 10.8 A)."""
    spacing: float = 0.9
    plateau: float = 10.0
    nl_cutoff: float = 10.8
    margin: float = 10.8
    outer_ext: int = 32
    alphabet: list = field(default_factory=lambda: list(range(1, 33)))


def dofs_modes(dofs6: np.ndarray, modes_rec: np.ndarray | None = None,
               modes_lig: np.ndarray | None = None) -> np.ndarray:
    """Packs (n,6) rigid DOFs plus mode amplitudes into (n,26) DOF_6D_Modes records."""
    n = dofs6.shape[0]
    out = np.zeros((n, DOF_MODES_WIDTH), dtype=np.float32)
    out[:, :6] = dofs6
    if modes_rec is not None:
        out[:, 6:6 + modes_rec.shape[1]] = modes_rec
    if modes_lig is not None:
        out[:, 16:16 + modes_lig.shape[1]] = modes_lig
    return out
