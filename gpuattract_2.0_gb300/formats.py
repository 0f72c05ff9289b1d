"""File formats on either side of the energy path, through libgbattract's C ABI
(include/gbattract_io.h).

Readers and writers keep gpuATTRACT 2.0's own file handling:
  read_pdb            readProteinFromPDB       src/fileIO/readFile.cpp:103-175
  read_params         readParamTableFromFile   src/fileIO/readFile.cpp:431-520
  read_alphabet       readGridAlphabetFromFile src/fileIO/readFile.cpp:901-926
  map_types           Configurator_6D::init    src/service/Configurator_6D.tpp:49-54
  read_dof/write_dof  readDOF, readDOFHeader   src/fileIO/readFile.cpp:579-651,747-871
  auto_pivot          Protein::auto_pivotize   src/model/Protein.tpp:145-157
  glob2rec            transformDOF_glob2rec    src/model/DOFTransform.cpp:35-90
  write_results       operator<< of Result_6D(_Modes), ATTRACT .score layout
  read_results        readResult               src/fileIO/readFile.cpp:653-745
  read_grid/write_grid  ATTRACT .grid          src/fileIO/grid_orig.cpp:85-484,
                                               src/fileIO/readFile.cpp:261-422
load_docking_inputs() strings them together the way Configurator_6D::init
(src/service/Configurator_6D.tpp:31-104) prepares a receptor/ligand run.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib
from .model import (FFPARAM_DTYPE, FELEC, DIELEC_CONSTANT, DIELEC_VARIABLE, GridSet, IntrplDesc,
                    NLDesc, ParamTable, Protein)

STREAM = 0     # GBA_RESULTS_STREAM
SCORE = 1      # GBA_RESULTS_SCORE


class DofHeaderC(C.Structure):
    _fields_ = [("auto_pivot", C.c_int32), ("centered_receptor", C.c_int32),
                ("centered_ligands", C.c_int32), ("num_pivots", C.c_uint32),
                ("pivots", (C.c_float * 3) * 16)]


class GridFileInfoC(C.Structure):
    _fields_ = [("gridspacing", C.c_double), ("gridextension", C.c_int32),
                ("plateaudis", C.c_double), ("neighbourdis", C.c_double),
                ("alphabet", C.c_uint8 * 99), ("ori", C.c_float * 3),
                ("inner_dim", C.c_int32 * 3), ("outer_dim", C.c_int32 * 3),
                ("natoms", C.c_int32), ("pivot", C.c_double * 3),
                ("architecture", C.c_uint16), ("nr_energrads", C.c_int32),
                ("nr_neighbours", C.c_int32)]


class IoError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbattract io error {code}: {msg}")
        self.code = code


_io = None


def _load():
    global _io
    if _io is not None:
        return _io
    lib = _lib.load()
    P, U32, SZ, I32 = C.c_void_p, C.c_uint32, C.c_size_t, C.c_int32
    s = C.c_char_p
    pu = C.POINTER(U32)
    sig = {
        "gba_io_last_error": ([], s),
        "gba_read_pdb": ([s, pu, P, P, P, U32], C.c_int),
        "gba_read_params": ([s, pu, P, U32, C.POINTER(I32), C.POINTER(C.c_float),
                             C.POINTER(C.c_float)], C.c_int),
        "gba_read_alphabet": ([s, pu, P, U32], C.c_int),
        "gba_map_types": ([P, U32, P, U32, P, P], C.c_int),
        "gba_read_dof": ([s, C.POINTER(DofHeaderC), pu, pu, P, P, SZ], C.c_int),
        "gba_write_dof": ([s, C.POINTER(DofHeaderC), U32, U32, P, P, P], C.c_int),
        "gba_auto_pivot": ([P, U32, P], C.c_int),
        "gba_dof_glob2rec": ([P, P, SZ, SZ, P, P, I32, I32], C.c_int),
        "gba_write_results": ([s, I32, I32, P, SZ, U32, U32], C.c_int),
        "gba_read_results": ([s, C.POINTER(SZ), pu, P, P, SZ, U32], C.c_int),
        "gba_grid_file_info_read": ([s, C.POINTER(GridFileInfoC)], C.c_int),
        "gba_read_grid_file": ([s, C.POINTER(_lib.IntrplDescC), P, C.POINTER(_lib.IntrplDescC), P,
                                C.POINTER(_lib.NLDescC), P, P], C.c_int),
        "gba_write_grid_file": ([s, C.POINTER(GridFileInfoC), P, C.POINTER(_lib.IntrplDescC), P,
                                 C.POINTER(_lib.IntrplDescC), P, C.POINTER(_lib.NLDescC), P, P, P],
                                C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _io = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise IoError(rc, _load().gba_io_last_error().decode())


def _b(path) -> bytes:
    return str(path).encode()


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- inputs --

def read_pdb(path) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Reduced PDB -> (xyz (3, n) float32, raw type (n,) uint32, charge (n,) float32)."""
    L = _load()
    n = C.c_uint32()
    _check(L.gba_read_pdb(_b(path), C.byref(n), None, None, None, 0))
    xyz = np.zeros((3, n.value), np.float32)
    t = np.zeros(n.value, np.uint32)
    q = np.zeros(n.value, np.float32)
    _check(L.gba_read_pdb(_b(path), C.byref(n), _p(xyz), _p(t), _p(q), n.value))
    return xyz, t, q


def read_params(path, dielec: int = DIELEC_VARIABLE, epsilon: float = 15.0) -> ParamTable:
    """attract.par -> ParamTable with SimParam's ffelec = FELEC / epsilon (as float)."""
    L = _load()
    T = C.c_uint32()
    shape = C.c_int32()
    _check(L.gba_read_params(_b(path), C.byref(T), None, 0, C.byref(shape), None, None))
    table = np.zeros(T.value * T.value, FFPARAM_DTYPE)
    _check(L.gba_read_params(_b(path), C.byref(T), _p(table), T.value * T.value, C.byref(shape),
                             None, None))
    ffelec = float(np.float32(FELEC / epsilon))
    return ParamTable(table=table, potshape=int(shape.value), dielec=dielec, ffelec=ffelec)


def read_alphabet(path) -> np.ndarray:
    L = _load()
    n = C.c_uint32()
    _check(L.gba_read_alphabet(_b(path), C.byref(n), None, 0))
    out = np.zeros(n.value, np.uint32)
    _check(L.gba_read_alphabet(_b(path), C.byref(n), _p(out), n.value))
    return out


def map_types(alphabet, types) -> tuple[np.ndarray, np.ndarray]:
    """(default-mapped types, grid channels) of the ligand, Configurator_6D.tpp:49-54."""
    a = np.ascontiguousarray(alphabet, np.uint32)
    t = np.ascontiguousarray(types, np.uint32)
    out_t = np.zeros_like(t)
    out_m = np.zeros_like(t)
    _check(_load().gba_map_types(_p(a), a.size, _p(t), t.size, _p(out_t), _p(out_m)))
    return out_t, out_m


# ----------------------------------------------------------------- DOFs --

@dataclass
class DofFile:
    """values: (structures, molecules, 16) float32 (ang xyz, pos xyz, extras);
    counts: (structures, molecules) values present on each line."""
    values: np.ndarray
    counts: np.ndarray
    auto_pivot: bool = True
    centered_receptor: bool = False
    centered_ligands: bool = False
    pivots: list = field(default_factory=list)

    @property
    def num_structures(self) -> int:
        return int(self.values.shape[0])

    @property
    def num_molecules(self) -> int:
        return int(self.values.shape[1])

    def dofs6(self, molecule: int) -> np.ndarray:
        """(n, 6) DOF_6D records {pos xyz, ang xyz} of one molecule (DOFConverter)."""
        v = self.values[:, molecule]
        return np.ascontiguousarray(np.concatenate([v[:, 3:6], v[:, 0:3]], axis=1), np.float32)


def read_dof(path) -> DofFile:
    L = _load()
    h = DofHeaderC()
    S, M = C.c_uint32(), C.c_uint32()
    _check(L.gba_read_dof(_b(path), C.byref(h), C.byref(S), C.byref(M), None, None, 0))
    vals = np.zeros((S.value, M.value, 16), np.float32)
    cnt = np.zeros((S.value, M.value), np.int32)
    _check(L.gba_read_dof(_b(path), C.byref(h), C.byref(S), C.byref(M), _p(vals), _p(cnt),
                          S.value * M.value))
    piv = [tuple(h.pivots[k][a] for a in range(3)) for k in range(h.num_pivots)]
    return DofFile(vals, cnt, bool(h.auto_pivot), bool(h.centered_receptor),
                   bool(h.centered_ligands), piv)


def write_dof(path, dof: DofFile, energies=None) -> None:
    h = DofHeaderC()
    h.auto_pivot = int(dof.auto_pivot)
    h.centered_receptor = int(dof.centered_receptor)
    h.centered_ligands = int(dof.centered_ligands)
    h.num_pivots = len(dof.pivots)
    for k, p in enumerate(dof.pivots):
        for a in range(3):
            h.pivots[k][a] = float(p[a])
    vals = np.ascontiguousarray(dof.values, np.float32)
    cnt = np.ascontiguousarray(dof.counts, np.int32)
    e = None if energies is None else np.ascontiguousarray(energies, np.float32)
    _check(_load().gba_write_dof(_b(path), C.byref(h), dof.num_structures, dof.num_molecules,
                                 _p(vals), _p(cnt), _p(e)))


def auto_pivot(xyz: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(xyz, np.float32)
    out = np.zeros(3, np.float32)
    _check(_load().gba_auto_pivot(_p(x), x.shape[1], _p(out)))
    return out


def glob2rec(dofs_rec: np.ndarray, dofs_lig: np.ndarray, pivot_rec, pivot_lig,
             centered_rec: bool, centered_lig: bool) -> tuple[np.ndarray, np.ndarray]:
    """transformDOF_glob2rec on (n, 6) or (n, 26) records; returns new arrays."""
    r = np.array(dofs_rec, np.float32, copy=True, order="C")
    lg = np.array(dofs_lig, np.float32, copy=True, order="C")
    pr = np.ascontiguousarray(pivot_rec, np.float32)
    pl = np.ascontiguousarray(pivot_lig, np.float32)
    _check(_load().gba_dof_glob2rec(_p(r), _p(lg), r.shape[0], r.shape[1] * 4, _p(pr), _p(pl),
                                    int(centered_rec), int(centered_lig)))
    return r, lg


# -------------------------------------------------------------- results --

def write_results(path, results: np.ndarray, n_modes_rec: int = 0, n_modes_lig: int = 0,
                  style: int = STREAM, append: bool = False) -> None:
    r = np.ascontiguousarray(results, np.float32)
    _check(_load().gba_write_results(_b(path), int(append), style, _p(r), r.shape[0],
                                     n_modes_rec, n_modes_lig))


def read_results(path) -> list:
    """readResult records: one float64 array per record (E, then gradient values)."""
    L = _load()
    n = C.c_size_t()
    w = C.c_uint32()
    _check(L.gba_read_results(_b(path), C.byref(n), C.byref(w), None, None, 0, 0))
    stride = max(1, w.value)
    out = np.zeros((n.value, stride), np.float64)
    cnt = np.zeros(n.value, np.int32)
    _check(L.gba_read_results(_b(path), C.byref(n), C.byref(w), _p(out), _p(cnt), n.value, stride))
    return [out[i, :cnt[i]].copy() for i in range(n.value)]


# ----------------------------------------------------------------- grids --

def _intrpl_c(d: IntrplDesc):
    c = _lib.IntrplDescC()
    c.numGrids = d.numGrids
    for a in range(3):
        c.dimN[a] = d.dimN[a]
        c.posMin[a] = d.posMin[a]
    c.gridSpacing = d.gridSpacing
    return c


def _nl_c(d: NLDesc):
    c = _lib.NLDescC()
    for a in range(3):
        c.dimN[a] = d.dimN[a]
        c.posMin[a] = d.posMin[a]
    c.gridSpacing = d.gridSpacing
    c.dPlateau = d.dPlateau
    c.numEl = d.numEl
    return c


def grid_file_info(path) -> GridFileInfoC:
    info = GridFileInfoC()
    _check(_load().gba_grid_file_info_read(_b(path), C.byref(info)))
    return info


def read_grid(path) -> tuple[GridSet, GridFileInfoC]:
    """ATTRACT .grid -> (GridSet in the file's absolute frame, header)."""
    L = _load()
    info = grid_file_info(path)
    ci, co, cn = _lib.IntrplDescC(), _lib.IntrplDescC(), _lib.NLDescC()
    C_ = 1 + sum(1 for a in info.alphabet if a)
    di = tuple(int(v) for v in info.inner_dim)
    do = tuple(int(v) for v in info.outer_dim)
    inner = np.zeros((C_, di[2], di[1], di[0], 4), np.float32)
    outer = np.zeros((C_, do[2], do[1], do[0], 4), np.float32)
    nlg = np.zeros((di[2], di[1], di[0], 2), np.uint32)
    nll = np.zeros(max(0, info.nr_neighbours), np.uint32)
    _check(L.gba_read_grid_file(_b(path), C.byref(ci), _p(inner), C.byref(co), _p(outer),
                                C.byref(cn), _p(nlg), _p(nll)))
    gs = GridSet(
        inner=IntrplDesc(ci.numGrids, tuple(ci.dimN), ci.gridSpacing, tuple(ci.posMin)),
        inner_data=inner,
        outer=IntrplDesc(co.numGrids, tuple(co.dimN), co.gridSpacing, tuple(co.posMin)),
        outer_data=outer,
        nl=NLDesc(tuple(cn.dimN), cn.gridSpacing, cn.dPlateau, tuple(cn.posMin), cn.numEl),
        nl_grid=nlg, nl_list=nll)
    return gs, info


def grid_header(grid: GridSet, alphabet, natoms: int, pivot=(0.0, 0.0, 0.0),
                neighbourdis: float = 10.8, gridextension: int = 32,
                architecture: int = 64) -> GridFileInfoC:
    """The .grid header describing a GridSet built with this library."""
    info = GridFileInfoC()
    info.gridspacing = float(np.float32(grid.inner.gridSpacing))
    info.gridextension = gridextension
    info.plateaudis = float(np.float32(grid.nl.dPlateau))
    info.neighbourdis = float(np.float32(neighbourdis))
    for t in alphabet:
        info.alphabet[int(t) - 1] = 1
    for a in range(3):
        info.ori[a] = grid.inner.posMin[a]
        info.inner_dim[a] = grid.inner.dimN[a]
        info.outer_dim[a] = grid.outer.dimN[a]
        info.pivot[a] = float(pivot[a])
    info.natoms = natoms
    info.architecture = architecture
    return info


def write_grid(path, grid: GridSet, alphabet, info: GridFileInfoC, rec_xyz=None) -> None:
    """write_std of a GridSet (channel c >= 1 holds type alphabet[c-1])."""
    a = np.ascontiguousarray(alphabet, np.uint32)
    ci, co, cn = _intrpl_c(grid.inner), _intrpl_c(grid.outer), _nl_c(grid.nl)
    x = None if rec_xyz is None else np.ascontiguousarray(rec_xyz, np.float32)
    _check(_load().gba_write_grid_file(
        _b(path), C.byref(info), _p(a), C.byref(ci), _p(np.ascontiguousarray(grid.inner_data)),
        C.byref(co), _p(np.ascontiguousarray(grid.outer_data)), C.byref(cn),
        _p(np.ascontiguousarray(grid.nl_grid)), _p(np.ascontiguousarray(grid.nl_list)), _p(x)))


def translate_grid(grid: GridSet, displ) -> GridSet:
    """GridUnion::translate: shift every origin by displ (float arithmetic)."""
    d = np.asarray(displ, np.float32)

    def sh(p):
        return tuple(float(np.float32(p[a]) + d[a]) for a in range(3))

    return GridSet(
        inner=IntrplDesc(grid.inner.numGrids, grid.inner.dimN, grid.inner.gridSpacing,
                         sh(grid.inner.posMin)),
        inner_data=grid.inner_data,
        outer=IntrplDesc(grid.outer.numGrids, grid.outer.dimN, grid.outer.gridSpacing,
                         sh(grid.outer.posMin)),
        outer_data=grid.outer_data,
        nl=NLDesc(grid.nl.dimN, grid.nl.gridSpacing, grid.nl.dPlateau, sh(grid.nl.posMin),
                  grid.nl.numEl),
        nl_grid=grid.nl_grid, nl_list=grid.nl_list)


# ------------------------------------------------------------ whole run --

@dataclass
class DockingInputs:
    rec: Protein
    lig: Protein
    grid: GridSet
    params: ParamTable
    dofs: np.ndarray           # (n, 6) ligand DOF_6D in the receptor frame
    pivots: tuple


def load_docking_inputs(dof_path, rec_pdb, lig_pdb, par_path, grid_path, alphabet_path,
                        dielec: str = "variable", epsilon: float = 15.0) -> DockingInputs:
    """Configurator_6D::init for a receptor/ligand pair
    (src/service/Configurator_6D.tpp:31-104): proteins, parameters and grid
    from their files, ligand types mapped by the receptor grid alphabet,
    pivots (auto or explicit), DOFs moved into the receptor frame, grid
    translated by -receptor pivot."""
    rxyz, rtype, rq = read_pdb(rec_pdb)
    lxyz, ltype, lq = read_pdb(lig_pdb)
    params = read_params(par_path, DIELEC_VARIABLE if dielec == "variable" else DIELEC_CONSTANT,
                         epsilon)
    grid, _ = read_grid(grid_path)
    alphabet = read_alphabet(alphabet_path)
    lt, lmapped = map_types(alphabet, ltype)
    dof = read_dof(dof_path)
    if dof.num_molecules != 2:
        raise ValueError("DOF file must describe exactly two molecules (receptor, ligand)")
    if dof.auto_pivot:
        if dof.pivots:
            raise ValueError("auto pivot specified, but explicit pivots are present")
        pr, pl = auto_pivot(rxyz), auto_pivot(lxyz)
    else:
        if len(dof.pivots) != 2:
            raise ValueError("no auto pivot, but the number of defined pivots is not 2")
        pr = np.asarray(dof.pivots[0], np.float32)
        pl = np.asarray(dof.pivots[1], np.float32)
    rxyz = (rxyz - pr[:, None]).astype(np.float32)
    lxyz = (lxyz - pl[:, None]).astype(np.float32)
    _, dl = glob2rec(dof.dofs6(0), dof.dofs6(1), pr, pl, dof.centered_receptor,
                     dof.centered_ligands)
    rec = Protein(xyz=rxyz, type=rtype, mapped=np.zeros_like(rtype), charge=rq)
    lig = Protein(xyz=lxyz, type=lt, mapped=lmapped, charge=lq)
    return DockingInputs(rec, lig, translate_grid(grid, -pr), params, dl, (pr, pl))
