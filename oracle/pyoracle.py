"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so) and of the
reference's own CPU path (oracle/_ref/libattract_ref.so, present only where
the reference tree was available at build time).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libattract_ref.so"


def _pkg():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import __graft_entry__
    return __graft_entry__.load_package()


class IntrplDescC(C.Structure):
    _fields_ = [("numGrids", C.c_uint32), ("dimN", C.c_uint32 * 3),
                ("gridSpacing", C.c_float), ("posMin", C.c_float * 3)]


class NLDescC(C.Structure):
    _fields_ = [("dimN", C.c_uint32 * 3), ("gridSpacing", C.c_float), ("dPlateau", C.c_float),
                ("posMin", C.c_float * 3), ("numEl", C.c_uint32)]


class OrcProtein(C.Structure):
    _fields_ = [("n", C.c_uint32), ("xyz", C.c_void_p), ("type", C.c_void_p),
                ("mapped", C.c_void_p), ("charge", C.c_void_p), ("n_modes", C.c_uint32),
                ("modes", C.c_void_p), ("mode_force", C.c_void_p)]


class OrcGrid(C.Structure):
    _fields_ = [("inner", IntrplDescC), ("inner_data", C.c_void_p),
                ("outer", IntrplDescC), ("outer_data", C.c_void_p),
                ("nl", NLDescC), ("nl_grid", C.c_void_p), ("nl_list", C.c_void_p)]


class OrcParams(C.Structure):
    _fields_ = [("num_types", C.c_uint32), ("table", C.c_void_p), ("potshape", C.c_int),
                ("dielec", C.c_int), ("ffelec", C.c_float)]


class OrcGridOpts(C.Structure):
    _fields_ = [("spacing", C.c_float), ("plateau", C.c_float), ("nl_cutoff", C.c_float),
                ("margin", C.c_float), ("outer_ext", C.c_uint32), ("n_alphabet", C.c_uint32),
                ("alphabet", C.c_uint32 * 99)]


STATS_DTYPE = np.dtype([("n_grid", "<u4"), ("n_grid_charged", "<u4"), ("n_nl", "<u4"),
                        ("n_nl_entries", "<u4"), ("n_pairs", "<u4"), ("n_rec_lookups", "<u4"),
                        ("abs_E", "<f8"), ("abs_F", "<f8"), ("abs_T", "<f8"), ("n_force_lim", "<u4"),
                        ("pad", "<u4")])

_orc = None
_ref = None


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def lib():
    global _orc
    if _orc is None:
        if not ORACLE_LIB.exists():
            raise ImportError(f"oracle not built: {ORACLE_LIB} (make -C oracle)")
        _orc = C.CDLL(str(ORACLE_LIB))
        for f in ("orc_energy_6d", "orc_energy_6d_f64", "orc_energy_6d_modes", "orc_energy_6d_modes_f64",
                  "orc_minimize_6d",
                  "orc_minimize_6d_modes", "orc_grid_layout", "orc_grid_build", "orc_grid_nl",
                  "orc_grid_voxels", "orc_pairwise_energy_f64"):
            getattr(_orc, f).restype = C.c_int
    return _orc


def ref_available() -> bool:
    return REF_LIB.exists()


def ref_root():
    """Root of the reference tree oracle/_ref was built from (None if absent)."""
    marker = HERE / "_ref" / "ref_root.txt"
    if not marker.exists():
        return None
    root = Path(marker.read_text().strip())
    return root if (root / "src").is_dir() else None


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise ImportError(f"reference CPU path not built: {REF_LIB} (oracle/build_ref.sh)")
        _ref = C.CDLL(str(REF_LIB))
        _ref.ref_last_error.restype = C.c_char_p
        for f in ("ref_energy_6d", "ref_energy_6d_modes", "ref_read_pdb", "ref_read_params"):
            getattr(_ref, f).restype = C.c_int
    return _ref


class _Keep:
    """Holds numpy arrays alive while their addresses sit in ctypes structs."""
    def __init__(self):
        self.arrs = []

    def __call__(self, a, dtype=None):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        self.arrs.append(a)
        return a.ctypes.data


def protein_c(p, keep: _Keep) -> OrcProtein:
    c = OrcProtein()
    c.n = p.n
    c.xyz = keep(p.xyz, np.float32)
    c.type = keep(p.type, np.uint32)
    c.mapped = keep(p.mapped, np.uint32)
    c.charge = keep(p.charge, np.float32)
    c.n_modes = p.n_modes
    c.modes = keep(p.modes, np.float32) if p.n_modes else None
    c.mode_force = keep(p.mode_force, np.float32) if p.n_modes else None
    return c


def _intrpl(d) -> IntrplDescC:
    c = IntrplDescC()
    c.numGrids = d.numGrids
    for a in range(3):
        c.dimN[a] = int(d.dimN[a])
        c.posMin[a] = float(d.posMin[a])
    c.gridSpacing = float(d.gridSpacing)
    return c


def grid_c(g, keep: _Keep) -> OrcGrid:
    c = OrcGrid()
    c.inner = _intrpl(g.inner)
    c.outer = _intrpl(g.outer)
    c.inner_data = keep(g.inner_data, np.float32)
    c.outer_data = keep(g.outer_data, np.float32)
    for a in range(3):
        c.nl.dimN[a] = int(g.nl.dimN[a])
        c.nl.posMin[a] = float(g.nl.posMin[a])
    c.nl.gridSpacing = float(g.nl.gridSpacing)
    c.nl.dPlateau = float(g.nl.dPlateau)
    c.nl.numEl = int(g.nl_list.shape[0])
    c.nl_grid = keep(g.nl_grid, np.uint32)
    c.nl_list = keep(g.nl_list if g.nl_list.size else np.zeros(1, np.uint32), np.uint32)
    return c


def params_c(t, keep: _Keep) -> OrcParams:
    c = OrcParams()
    c.num_types = t.num_types
    c.table = keep(t.table)
    c.potshape = t.potshape
    c.dielec = t.dielec
    c.ffelec = float(t.ffelec)
    return c


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


def energy_6d(rec, lig, grid, params, dofs, stats: bool = False, nthreads: int = 0):
    """FP32 rigid energies (n, 7) [+ per-pose stats] from the restatement."""
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 7), dtype=np.float32)
    st = np.zeros(n, dtype=STATS_DTYPE) if stats else None
    R, L, G, P = protein_c(rec, k), protein_c(lig, k), grid_c(grid, k), params_c(params, k)
    _check(lib().orc_energy_6d(C.byref(R), C.byref(L), C.byref(G), C.byref(P), _p(dofs),
                               C.c_size_t(n), _p(out), _p(st), nthreads), "orc_energy_6d")
    return (out, st) if stats else out


def energy_6d_f64(rec, lig, grid, params, dofs, nthreads: int = 0):
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 7), dtype=np.float64)
    R, L, G, P = protein_c(rec, k), protein_c(lig, k), grid_c(grid, k), params_c(params, k)
    _check(lib().orc_energy_6d_f64(C.byref(R), C.byref(L), C.byref(G), C.byref(P), _p(dofs),
                                   C.c_size_t(n), _p(out), nthreads), "orc_energy_6d_f64")
    return out


def energy_6d_modes_f64(rec, lig, grid_rec, grid_lig, params, dofs, nthreads: int = 0):
    """The normal-mode evaluation in FP64 throughout: (n, 27) float64."""
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 27), dtype=np.float64)
    R, L = protein_c(rec, k), protein_c(lig, k)
    GR, GL, P = grid_c(grid_rec, k), grid_c(grid_lig, k), params_c(params, k)
    _check(lib().orc_energy_6d_modes_f64(C.byref(R), C.byref(L), C.byref(GR), C.byref(GL),
                                         C.byref(P), _p(dofs), C.c_size_t(n), _p(out), nthreads),
           "orc_energy_6d_modes_f64")
    return out


def energy_6d_modes(rec, lig, grid_rec, grid_lig, params, dofs, stats: bool = False,
                    nthreads: int = 0):
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 27), dtype=np.float32)
    st = np.zeros(n, dtype=STATS_DTYPE) if stats else None
    R, L = protein_c(rec, k), protein_c(lig, k)
    GR, GL, P = grid_c(grid_rec, k), grid_c(grid_lig, k), params_c(params, k)
    _check(lib().orc_energy_6d_modes(C.byref(R), C.byref(L), C.byref(GR), C.byref(GL),
                                     C.byref(P), _p(dofs), C.c_size_t(n), _p(out), _p(st),
                                     nthreads), "orc_energy_6d_modes")
    return (out, st) if stats else out


def minimize_6d(rec, lig, grid, params, dofs, max_fun_eval: int, nthreads: int = 0):
    """VA13 per pose: (last state (n,6), last result (n,7), evaluations (n,))."""
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    st = np.zeros((n, 6), np.float32)
    res = np.zeros((n, 7), np.float32)
    nev = np.zeros(n, np.int32)
    R, L, G, P = protein_c(rec, k), protein_c(lig, k), grid_c(grid, k), params_c(params, k)
    _check(lib().orc_minimize_6d(C.byref(R), C.byref(L), C.byref(G), C.byref(P), _p(dofs),
                                 C.c_size_t(n), max_fun_eval, _p(st), _p(res), _p(nev), nthreads),
           "orc_minimize_6d")
    return st, res, nev


def minimize_6d_modes(rec, lig, grid_rec, grid_lig, params, dofs, max_fun_eval: int,
                      nthreads: int = 0):
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    st = np.zeros((n, 26), np.float32)
    res = np.zeros((n, 27), np.float32)
    nev = np.zeros(n, np.int32)
    R, L = protein_c(rec, k), protein_c(lig, k)
    GR, GL, P = grid_c(grid_rec, k), grid_c(grid_lig, k), params_c(params, k)
    _check(lib().orc_minimize_6d_modes(C.byref(R), C.byref(L), C.byref(GR), C.byref(GL),
                                       C.byref(P), _p(dofs), C.c_size_t(n), max_fun_eval,
                                       _p(st), _p(res), _p(nev), nthreads), "orc_minimize_6d_modes")
    return st, res, nev


def grid_opts_c(opt) -> OrcGridOpts:
    c = OrcGridOpts()
    c.spacing, c.plateau, c.nl_cutoff, c.margin = opt.spacing, opt.plateau, opt.nl_cutoff, opt.margin
    c.outer_ext = opt.outer_ext
    c.n_alphabet = len(opt.alphabet)
    for i, t in enumerate(opt.alphabet):
        c.alphabet[i] = int(t)
    return c


def build_grid(rec, params, opt, nthreads: int = 0):
    """CPU grid builder (the device builder's FP32 arithmetic and summation order) -> gbattract.GridSet."""
    m = _pkg().model
    k = _Keep()
    R, P, O = protein_c(rec, k), params_c(params, k), grid_opts_c(opt)
    inner, outer, nl = IntrplDescC(), IntrplDescC(), NLDescC()
    _check(lib().orc_grid_layout(C.byref(R), C.byref(O), C.byref(inner), C.byref(outer),
                                 C.byref(nl)), "orc_grid_layout")
    di = np.zeros((inner.numGrids, inner.dimN[2], inner.dimN[1], inner.dimN[0], 4), np.float32)
    do = np.zeros((outer.numGrids, outer.dimN[2], outer.dimN[1], outer.dimN[0], 4), np.float32)
    ng = np.zeros((nl.dimN[2], nl.dimN[1], nl.dimN[0], 2), np.uint32)
    cap = int(ng.shape[0] * ng.shape[1] * ng.shape[2]) * 16
    while True:
        lst = np.zeros(max(cap, 1), np.uint32)
        rc = lib().orc_grid_build(C.byref(R), C.byref(P), C.byref(O), C.byref(inner), _p(di),
                                  C.byref(outer), _p(do), C.byref(nl), _p(ng), _p(lst),
                                  C.c_size_t(cap), nthreads)
        if rc == 0:
            break
        if nl.numEl > cap:
            cap = int(nl.numEl)
            continue
        _check(rc, "orc_grid_build")
    to_i = lambda d: m.IntrplDesc(d.numGrids, tuple(d.dimN), d.gridSpacing, tuple(d.posMin))
    nld = m.NLDesc(tuple(nl.dimN), nl.gridSpacing, nl.dPlateau, tuple(nl.posMin), nl.numEl)
    return m.GridSet(to_i(inner), di, to_i(outer), do, nld, ng, lst[:nl.numEl].copy())


def grid_layout(rec, opt):
    """Descriptors (inner, outer, NL) the builders give receptor `rec`."""
    m = _pkg().model
    k = _Keep()
    R, O = protein_c(rec, k), grid_opts_c(opt)
    inner, outer, nl = IntrplDescC(), IntrplDescC(), NLDescC()
    _check(lib().orc_grid_layout(C.byref(R), C.byref(O), C.byref(inner), C.byref(outer),
                                 C.byref(nl)), "orc_grid_layout")
    to_i = lambda d: m.IntrplDesc(d.numGrids, tuple(d.dimN), d.gridSpacing, tuple(d.posMin))
    return to_i(inner), to_i(outer), nl


def build_grid_nl(rec, opt, nthreads: int = 0):
    """Neighbour-list part of build_grid alone: (NLDesc, nl_grid, nl_list)."""
    m = _pkg().model
    k = _Keep()
    R, O = protein_c(rec, k), grid_opts_c(opt)
    _, _, nl = grid_layout(rec, opt)
    ng = np.zeros((nl.dimN[2], nl.dimN[1], nl.dimN[0], 2), np.uint32)
    cap = int(ng.shape[0] * ng.shape[1] * ng.shape[2]) * 16
    while True:
        lst = np.zeros(max(cap, 1), np.uint32)
        rc = lib().orc_grid_nl(C.byref(R), C.byref(O), C.byref(nl), _p(ng), _p(lst), C.c_size_t(cap),
                               nthreads)
        if rc == 0:
            break
        if nl.numEl > cap:
            cap = int(nl.numEl)
            continue
        _check(rc, "orc_grid_nl")
    nld = m.NLDesc(tuple(nl.dimN), nl.gridSpacing, nl.dPlateau, tuple(nl.posMin), nl.numEl)
    return nld, ng, lst[:nl.numEl].copy()


def grid_voxels(rec, params, opt, desc, voxels, nthreads: int = 0):
    """Potentials of build_grid at the given linear voxel indices of the grid
    `desc` (an IntrplDesc): (len(voxels), numGrids, 4) float32."""
    k = _Keep()
    R, P, O = protein_c(rec, k), params_c(params, k), grid_opts_c(opt)
    d = _intrpl(desc)
    v = np.ascontiguousarray(voxels, np.uint64)
    out = np.zeros((len(v), desc.numGrids, 4), np.float32)
    _check(lib().orc_grid_voxels(C.byref(R), C.byref(P), C.byref(O), C.byref(d), _p(v), C.c_size_t(len(v)),
                                 _p(out), nthreads), "orc_grid_voxels")
    return out


class exact_sincos:
    """Context manager: inside it the FP32 oracle takes correctly rounded
    sin/cos ((float)sin((double)x)) instead of the C library's sinf/cosf,
    whose last-ulp rounding the C standard leaves to the implementation.  A
    difference between the two is the only input the device kernels (which
    compute correctly rounded sin/cos) cannot share with the reference."""

    def __enter__(self):
        lib().orc_set_exact_sincos(1)
        return self

    def __exit__(self, *a):
        lib().orc_set_exact_sincos(0)


def libm_sincos_rounds_exactly(angles) -> np.ndarray:
    """Per row of float32 angles: True when this host's sinf/cosf return the
    correctly rounded value for every angle of the row."""
    import ctypes.util
    m = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    m.sinf.restype = m.cosf.restype = C.c_float
    m.sinf.argtypes = m.cosf.argtypes = [C.c_float]
    a = np.asarray(angles, np.float32)
    ok = np.ones(a.shape[0], bool)
    for i, row in enumerate(a):
        for x in row:
            x = float(x)
            if (np.float32(m.sinf(x)) != np.float32(np.sin(np.float64(np.float32(x)))) or
                    np.float32(m.cosf(x)) != np.float32(np.cos(np.float64(np.float32(x))))):
                ok[i] = False
                break
    return ok


def pose_errors(got, ref, st):
    """Per-pose scaled errors of (E, force vector, torque vector): |d| over
    max(|ref|, 0.05 S), S the sum of the magnitudes of the terms the oracle
    added (st from energy_6d(..., stats=True)); the floor bounds the FP32
    summation error of sums that cancel."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    eE = np.abs(got[:, 0] - ref[:, 0]) / np.maximum(np.abs(ref[:, 0]), 0.05 * st["abs_E"] + 1e-30)
    eF = np.linalg.norm(got[:, 1:4] - ref[:, 1:4], axis=1) / np.maximum(
        np.linalg.norm(ref[:, 1:4], axis=1), 0.05 * st["abs_F"] + 1e-30)
    eT = np.linalg.norm(got[:, 4:7] - ref[:, 4:7], axis=1) / np.maximum(
        np.linalg.norm(ref[:, 4:7], axis=1), 0.05 * st["abs_T"] + 1e-30)
    return eE, eF, eT


def parity_stats(got, ref, st, ref64=None):
    """Summary of a GPU result against the FP32 oracle (and the FP64 one):
    the largest scaled error (pose_errors), the fractions of poses within
    1e-4 of the bare relative error |d| / |ref| (no floor), and the error of
    both FP32 results against FP64 on the energy, |d| / max(|E64|, 0.05 S)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    eE, eF, eT = pose_errors(got, ref, st)
    bare = lambda d, r: d <= 1e-4 * r
    bE = bare(np.abs(got[:, 0] - ref[:, 0]), np.abs(ref[:, 0]))
    bF = bare(np.linalg.norm(got[:, 1:4] - ref[:, 1:4], axis=1), np.linalg.norm(ref[:, 1:4], axis=1))
    bT = bare(np.linalg.norm(got[:, 4:7] - ref[:, 4:7], axis=1), np.linalg.norm(ref[:, 4:7], axis=1))
    out = {"poses": int(len(got)),
           "max_scaled_err": float(max(eE.max(), eF.max(), eT.max())),
           "frac_within_1e-4_bare": float(np.mean(bE & bF & bT)),
           "frac_within_1e-4_bare_E": float(np.mean(bE)),
           "frac_within_1e-4_bare_F": float(np.mean(bF)),
           "frac_within_1e-4_bare_T": float(np.mean(bT))}
    if ref64 is not None:
        r64 = np.asarray(ref64, np.float64)
        den = np.maximum(np.abs(r64[:, 0]), 0.05 * st["abs_E"] + 1e-30)
        g64 = np.abs(got[:, 0] - r64[:, 0]) / den
        o64 = np.abs(ref[:, 0] - r64[:, 0]) / den
        out.update({"fp64_err_median": float(np.median(g64)), "fp64_err_max": float(g64.max()),
                    "oracle_fp32_fp64_err_median": float(np.median(o64)),
                    "oracle_fp32_fp64_err_max": float(o64.max())})
    return out


def mode_gradient_errors(got, ref, Mr: int, Ml: int) -> np.ndarray:
    """Per pose (finite in ref) and side, |g - r| / max(|r|, 1e-3 max |r|) of
    the receptor and ligand mode-gradient vectors (Result_6D_Modes columns
    7.. and 17..)."""
    errs = []
    for lo, M in ((7, Mr), (17, Ml)):
        g = np.asarray(got, np.float64)[:, lo:lo + M]
        r = np.asarray(ref, np.float64)[:, lo:lo + M]
        fin = np.all(np.isfinite(r), axis=1) & np.all(np.isfinite(g), axis=1)
        g, r = g[fin], r[fin]
        if len(r) == 0:
            continue
        nr = np.linalg.norm(r, axis=1)
        errs.append(np.linalg.norm(g - r, axis=1) / np.maximum(nr, 1e-3 * nr.max() + 1e-30))
    return np.concatenate(errs) if errs else np.zeros(1)


def modes_parity_stats(got, ref, st, ref64, Mr: int, Ml: int) -> dict:
    """parity_stats of the rigid part of Result_6D_Modes (energy, force,
    torque) over the poses finite in the FP32 oracle, plus the mode
    gradients' errors against the FP32 oracle and of both FP32 results
    against the FP64 one."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    fin = np.isfinite(ref).all(axis=1) & np.isfinite(got).all(axis=1)
    out = parity_stats(got[fin, :7], ref[fin, :7], st[fin], np.asarray(ref64)[fin, :7])
    out["poses_finite"] = int(fin.sum())
    m32 = mode_gradient_errors(got[fin], ref[fin], Mr, Ml)
    g64 = mode_gradient_errors(got[fin], np.asarray(ref64)[fin], Mr, Ml)
    o64 = mode_gradient_errors(ref[fin], np.asarray(ref64)[fin], Mr, Ml)
    out.update({"mode_grad_max_err": float(m32.max()),
                "mode_grad_fp64_err_median": float(np.median(g64)), "mode_grad_fp64_err_max": float(g64.max()),
                "oracle_mode_grad_fp64_err_median": float(np.median(o64)),
                "oracle_mode_grad_fp64_err_max": float(o64.max())})
    return out


def minimization_stats(a, b, tol: float = 1e-3) -> dict:
    """Symmetric comparison of two sets of minimized results (column 0 = E)
    over the poses finite in both: the fraction within tol relative
    (|Ea - Eb| <= tol max(|Eb|, 1e-3)), the fraction where a ended at least as
    low as b (Ea <= Eb + tol |Eb|) and the converse, and the 10/25/50/75/90th
    percentiles of both."""
    ea = np.asarray(a, np.float64)[:, 0]
    eb = np.asarray(b, np.float64)[:, 0]
    fin = np.isfinite(ea) & np.isfinite(eb)
    ea, eb = ea[fin], eb[fin]
    den = np.maximum(np.abs(eb), 1e-3)
    q = [10, 25, 50, 75, 90]
    return {"poses": int(fin.sum()),
            "within_tol": float(np.mean(np.abs(ea - eb) / den <= tol)),
            "a_at_least_as_low": float(np.mean(ea <= eb + tol * den)),
            "b_at_least_as_low": float(np.mean(eb <= ea + tol * den)),
            "quantiles_pct": q,
            "a_quantiles": [float(x) for x in np.percentile(ea, q)],
            "b_quantiles": [float(x) for x in np.percentile(eb, q)],
            "a_mean": float(ea.mean()), "b_mean": float(eb.mean())}


def pairwise_energy_f64(rec, lig, q_rec, q_lig, r0, eps, ipon, dielec, ffelec, cutoff, dofs6,
                        ref_dofs6=None, grad: bool = False):
    """FP64 pairwise energies (n,) [and analytic dE/dDOF (n, 6), (pos, ang)]."""
    k = _Keep()
    R, L = protein_c(rec, k), protein_c(lig, k)
    dofs6 = np.ascontiguousarray(dofs6, np.float64)
    n = dofs6.shape[0]
    out = np.zeros(n, np.float64)
    g = np.zeros((n, 6), np.float64) if grad else None
    ref = None if ref_dofs6 is None else np.ascontiguousarray(ref_dofs6, np.float64)
    T = r0.shape[0]
    _check(lib().orc_pairwise_energy_f64(
        C.byref(R), C.byref(L), C.c_void_p(k(q_rec, np.float64)), C.c_void_p(k(q_lig, np.float64)), T,
        C.c_void_p(k(r0, np.float64)), C.c_void_p(k(eps, np.float64)), C.c_void_p(k(ipon, np.int32)),
        int(dielec), C.c_double(ffelec), C.c_double(cutoff), _p(dofs6), _p(ref), C.c_size_t(n),
        _p(out), _p(g)), "orc_pairwise_energy_f64")
    return (out, g) if grad else out


# ---- the reference's own CPU path ------------------------------------------

def ref_energy_6d(rec, lig, grid, params, dofs, nworkers: int = 2, item_size: int = 100):
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 7), dtype=np.float32)
    R, L, G, P = protein_c(rec, k), protein_c(lig, k), grid_c(grid, k), params_c(params, k)
    rc = ref_lib().ref_energy_6d(C.byref(R), C.byref(L), C.byref(G), C.byref(P), _p(dofs),
                                 C.c_size_t(n), _p(out), nworkers, item_size)
    if rc != 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    return out


def ref_energy_6d_modes(rec, lig, grid_rec, grid_lig, params, dofs, nworkers: int = 2,
                        item_size: int = 100):
    k = _Keep()
    dofs = np.ascontiguousarray(dofs, dtype=np.float32)
    n = dofs.shape[0]
    out = np.zeros((n, 27), dtype=np.float32)
    R, L = protein_c(rec, k), protein_c(lig, k)
    GR, GL, P = grid_c(grid_rec, k), grid_c(grid_lig, k), params_c(params, k)
    rc = ref_lib().ref_energy_6d_modes(C.byref(R), C.byref(L), C.byref(GR), C.byref(GL),
                                       C.byref(P), _p(dofs), C.c_size_t(n), _p(out), nworkers,
                                       item_size)
    if rc != 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    return out


def ref_read_pdb(path: str, default_map: bool = True):
    """(xyz (3,n), type, charge) through the reference's reduced-PDB reader."""
    n = ref_lib().ref_read_pdb(str(path).encode(), int(default_map), None, None, None, 0)
    if n < 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    xyz = np.zeros((3, n), np.float32)
    t = np.zeros(n, np.uint32)
    q = np.zeros(n, np.float32)
    ref_lib().ref_read_pdb(str(path).encode(), int(default_map), _p(xyz), _p(t), _p(q), n)
    return xyz, t, q


def ref_read_params(path: str):
    """(table as FFPARAM records, potshape) through the reference's attract.par reader."""
    ps = C.c_int()
    T = ref_lib().ref_read_params(str(path).encode(), None, 0, C.byref(ps))
    if T < 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    m = _pkg().model
    tab = np.zeros(T * T, m.FFPARAM_DTYPE)
    ref_lib().ref_read_params(str(path).encode(), _p(tab), T, C.byref(ps))
    return tab, ps.value


# ---- file formats through the reference's own readers / writers ----------

def _ref_fn(name, restype=C.c_int):
    f = getattr(ref_lib(), name)
    f.restype = restype
    return f


def ref_read_dof(path):
    """(values (S, M, 16), counts (S, M), header dict) via readDOF/readDOFHeader."""
    f = _ref_fn("ref_read_dof")
    M = C.c_int32()
    hdr = np.zeros(4, np.int32)
    piv = np.zeros((16, 3), np.float32)
    S = f(str(path).encode(), None, None, C.c_long(0), C.byref(M), _p(hdr), _p(piv))
    if S < 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    vals = np.zeros((S, M.value, 16), np.float32)
    cnt = np.zeros((S, M.value), np.int32)
    f(str(path).encode(), _p(vals), _p(cnt), C.c_long(S * M.value), C.byref(M), _p(hdr), _p(piv))
    h = dict(auto_pivot=bool(hdr[0]), centered_receptor=bool(hdr[1]),
             centered_ligands=bool(hdr[2]), pivots=[tuple(piv[k]) for k in range(hdr[3])])
    return vals, cnt, h


def ref_read_results(path, stride: int = 64):
    f = _ref_fn("ref_read_results", C.c_long)
    n = f(str(path).encode(), None, None, C.c_long(0), stride)
    if n < 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    out = np.zeros((n, stride), np.float64)
    cnt = np.zeros(n, np.int32)
    f(str(path).encode(), _p(out), _p(cnt), C.c_long(n), stride)
    return [out[i, :cnt[i]].copy() for i in range(n)]


def ref_write_results(path, results, n_modes_rec: int = 0, n_modes_lig: int = 0):
    r = np.ascontiguousarray(results, np.float32)
    if _ref_fn("ref_write_results")(str(path).encode(), _p(r), C.c_long(r.shape[0]),
                                    n_modes_rec, n_modes_lig) != 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())


def ref_glob2rec(dofs_rec, dofs_lig, pivot_rec, pivot_lig, centered_rec, centered_lig):
    r = np.array(dofs_rec, np.float32, copy=True, order="C")
    lg = np.array(dofs_lig, np.float32, copy=True, order="C")
    pr = np.ascontiguousarray(pivot_rec, np.float32)
    pl = np.ascontiguousarray(pivot_lig, np.float32)
    _ref_fn("ref_glob2rec")(_p(r), _p(lg), C.c_long(r.shape[0]), _p(pr), _p(pl),
                            int(centered_rec), int(centered_lig))
    return r, lg


def ref_auto_pivot(xyz):
    x = np.ascontiguousarray(xyz, np.float32)
    out = np.zeros(3, np.float32)
    _ref_fn("ref_auto_pivot")(_p(x), C.c_long(x.shape[1]), _p(out))
    return out


def ref_map_types(alphabet_path, types):
    t = np.ascontiguousarray(types, np.uint32)
    ot, om = np.zeros_like(t), np.zeros_like(t)
    alpha = np.zeros(128, np.uint32)
    n = _ref_fn("ref_map_types")(str(alphabet_path).encode(), _p(t), C.c_long(t.size), _p(ot),
                                 _p(om), _p(alpha), 128)
    if n < 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    return ot, om, alpha[:n].copy()


def ref_read_grid_file(path, info):
    """readGridFromGridFile<float>: (inner desc, inner, outer desc, outer, nl desc,
    nl_grid, nl_list, dPlateau2); buffers sized from the .grid header `info`."""
    from gbattract import _lib
    C_ = 1 + sum(1 for a in info.alphabet if a)
    di = [int(v) for v in info.inner_dim]
    do = [int(v) for v in info.outer_dim]
    inner = np.zeros((C_, di[2], di[1], di[0], 4), np.float32)
    outer = np.zeros((C_, do[2], do[1], do[0], 4), np.float32)
    nlg = np.zeros((di[2], di[1], di[0], 2), np.uint32)
    nll = np.zeros(max(1, info.nr_neighbours), np.uint32)
    ci, co, cn = _lib.IntrplDescC(), _lib.IntrplDescC(), _lib.NLDescC()
    dp2 = C.c_float()
    rc = _ref_fn("ref_read_grid_file")(
        str(path).encode(), C.byref(ci), _p(inner), C.c_long(inner.size), C.byref(co), _p(outer),
        C.c_long(outer.size), C.byref(cn), _p(nlg), C.c_long(nlg.size // 2), _p(nll),
        C.c_long(info.nr_neighbours), C.byref(dp2))
    if rc != 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
    return ci, inner, co, outer, cn, nlg, nll[:info.nr_neighbours], dp2.value


def ref_write_grid_file(path, grid, alphabet, info, rec_xyz=None):
    """attract::Grid::write_std of a GridSet (the reference's own writer)."""
    from gbattract import _lib, formats
    a = np.ascontiguousarray(alphabet, np.uint32)
    ci, co, cn = formats._intrpl_c(grid.inner), formats._intrpl_c(grid.outer), formats._nl_c(grid.nl)
    x = None if rec_xyz is None else np.ascontiguousarray(rec_xyz, np.float32)
    rc = _ref_fn("ref_write_grid_file")(
        str(path).encode(), C.byref(info), _p(a), C.byref(ci), _p(np.ascontiguousarray(grid.inner_data)),
        C.byref(co), _p(np.ascontiguousarray(grid.outer_data)), C.byref(cn),
        _p(np.ascontiguousarray(grid.nl_grid)), _p(np.ascontiguousarray(grid.nl_list)), _p(x))
    if rc != 0:
        raise RuntimeError(ref_lib().ref_last_error().decode())
