"""GbaContext: the Python face of libgbattract's C ABI.

A context owns device copies of proteins, grids and parameter tables (what
the reference's DataManager + DeviceDataConfigurator hold per device,
src/server/DataManager.cpp:23-101, src/server/DeviceDataConfigurator.tpp:28-362)
and evaluates poses through the fused kernels.  Pose arrays may be numpy
arrays (host) or torch tensors (host or CUDA); results come back in the same
kind of array.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .model import (DOF_MODES_WIDTH, DOF_WIDTH, RESULT_MODES_WIDTH, RESULT_WIDTH, GridOptions,
                    GridSet, IntrplDesc, NLDesc, ParamTable, Protein)


def _intrpl_c(d: IntrplDesc) -> _lib.IntrplDescC:
    c = _lib.IntrplDescC()
    c.numGrids = d.numGrids
    for a in range(3):
        c.dimN[a] = int(d.dimN[a])
        c.posMin[a] = float(d.posMin[a])
    c.gridSpacing = float(d.gridSpacing)
    return c


def _nl_c(d: NLDesc) -> _lib.NLDescC:
    c = _lib.NLDescC()
    for a in range(3):
        c.dimN[a] = int(d.dimN[a])
        c.posMin[a] = float(d.posMin[a])
    c.gridSpacing = float(d.gridSpacing)
    c.dPlateau = float(d.dPlateau)
    c.numEl = int(d.numEl)
    return c


def grid_opts_c(opt: GridOptions) -> _lib.GridBuildOptsC:
    c = _lib.GridBuildOptsC()
    c.spacing = opt.spacing
    c.plateau = opt.plateau
    c.nl_cutoff = opt.nl_cutoff
    c.margin = opt.margin
    c.outer_ext = opt.outer_ext
    c.n_alphabet = len(opt.alphabet)
    for i, t in enumerate(opt.alphabet):
        c.alphabet[i] = int(t)
    return c


def _is_torch(a) -> bool:
    return hasattr(a, "data_ptr") and hasattr(a, "is_cuda")


def _alloc_like(a, shape):
    if _is_torch(a):
        import torch
        return torch.empty(shape, dtype=torch.float32, device=a.device)
    return np.empty(shape, dtype=np.float32)


def _check_poses(a, width: int, what: str):
    if _is_torch(a):
        import torch
        if a.dtype != torch.float32 or a.dim() != 2 or a.shape[1] != width or not a.is_contiguous():
            raise ValueError(f"{what}: expected a contiguous float32 (n, {width}) tensor")
        return a
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != width:
        raise ValueError(f"{what}: expected (n, {width}) poses")
    return a


class GbaContext:
    """Device context; see include/gbattract.h for the semantics of each call."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.gba_create(device, C.byref(h))
        if rc != _lib.GBA_OK:
            raise _lib.GbaError(rc, self.lib.gba_last_error(None).decode())
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.gba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        _lib.check(self.h, rc)

    # ---- uploads -------------------------------------------------------------
    def upload_protein(self, p: Protein) -> int:
        out = C.c_uint32()
        modes = p.modes if p.modes is not None else None
        self._check(self.lib.gba_upload_protein(
            self.h, p.n, _lib.ptr(p.xyz), _lib.ptr(p.type), _lib.ptr(p.mapped), _lib.ptr(p.charge),
            p.n_modes, _lib.ptr(modes), _lib.ptr(p.mode_force), C.byref(out)))
        return out.value

    def upload_grid(self, g: GridSet) -> int:
        out = C.c_uint32()
        inner, outer, nl = _intrpl_c(g.inner), _intrpl_c(g.outer), _nl_c(g.nl)
        nl.numEl = int(g.nl_list.shape[0])
        self._check(self.lib.gba_upload_grid(
            self.h, C.byref(inner), _lib.ptr(np.ascontiguousarray(g.inner_data)), C.byref(outer),
            _lib.ptr(np.ascontiguousarray(g.outer_data)), C.byref(nl),
            _lib.ptr(np.ascontiguousarray(g.nl_grid)),
            _lib.ptr(np.ascontiguousarray(g.nl_list)) if g.nl_list.size else None, C.byref(out)))
        return out.value

    def upload_params(self, t: ParamTable) -> int:
        out = C.c_uint32()
        tab = np.ascontiguousarray(t.table)
        self._check(self.lib.gba_upload_params(self.h, t.num_types, _lib.ptr(tab), t.potshape,
                                               t.dielec, float(t.ffelec), C.byref(out)))
        return out.value

    def release(self, item: int):
        self._check(self.lib.gba_release(self.h, item))

    # ---- grid builder --------------------------------------------------------
    def build_grid(self, rec: int, params: int, opt: GridOptions | None = None) -> int:
        """Builds inner/outer/NL grids of receptor `rec` on the device."""
        opt = opt or GridOptions()
        o = grid_opts_c(opt)
        out = C.c_uint32()
        self._check(self.lib.gba_build_grid(self.h, rec, params, C.byref(o), C.byref(out)))
        return out.value

    def download_grid(self, grid: int) -> GridSet:
        """Copies a device grid back into a host GridSet."""
        i, o, n = _lib.IntrplDescC(), _lib.IntrplDescC(), _lib.NLDescC()
        self._check(self.lib.gba_grid_info(self.h, grid, C.byref(i), C.byref(o), C.byref(n)))
        inner = IntrplDesc(i.numGrids, tuple(i.dimN), i.gridSpacing, tuple(i.posMin))
        outer = IntrplDesc(o.numGrids, tuple(o.dimN), o.gridSpacing, tuple(o.posMin))
        nld = NLDesc(tuple(n.dimN), n.gridSpacing, n.dPlateau, tuple(n.posMin), n.numEl)
        di = np.empty((inner.numGrids, inner.dimN[2], inner.dimN[1], inner.dimN[0], 4), np.float32)
        do = np.empty((outer.numGrids, outer.dimN[2], outer.dimN[1], outer.dimN[0], 4), np.float32)
        ng = np.empty((nld.dimN[2], nld.dimN[1], nld.dimN[0], 2), np.uint32)
        nlst = np.empty(max(1, n.numEl), np.uint32)
        self._check(self.lib.gba_download_grid(self.h, grid, _lib.ptr(di), _lib.ptr(do),
                                               _lib.ptr(ng), _lib.ptr(nlst)))
        return GridSet(inner, di, outer, do, nld, ng, nlst[:n.numEl])

    # ---- evaluation ----------------------------------------------------------
    def energy_6d(self, rec: int, lig: int, grid: int, params: int, dofs, out=None,
                  stream=None):
        """One energy+gradient evaluation per pose; returns (n, 7) results."""
        dofs = _check_poses(dofs, DOF_WIDTH, "energy_6d")
        n = dofs.shape[0]
        if out is None:
            out = _alloc_like(dofs, (n, RESULT_WIDTH))
        self._check(self.lib.gba_energy_6d(self.h, rec, lig, grid, params, _lib.ptr(dofs), n,
                                           _lib.ptr(out), stream))
        return out

    def energy_6d_modes(self, rec: int, lig: int, grid_rec: int, grid_lig: int, params: int,
                        dofs, out=None, stream=None):
        """Normal-mode variant; dofs (n, 26) -> results (n, 27)."""
        dofs = _check_poses(dofs, DOF_MODES_WIDTH, "energy_6d_modes")
        n = dofs.shape[0]
        if out is None:
            out = _alloc_like(dofs, (n, RESULT_MODES_WIDTH))
        self._check(self.lib.gba_energy_6d_modes(self.h, rec, lig, grid_rec, grid_lig, params,
                                                 _lib.ptr(dofs), n, _lib.ptr(out), stream))
        return out

    # ---- minimization ----------------------------------------------------------
    def _min_outputs(self, dofs):
        n = dofs.shape[0]
        if _is_torch(dofs):
            import torch
            return (torch.empty((n, DOF_WIDTH), dtype=torch.float32, device=dofs.device),
                    torch.empty((n, RESULT_WIDTH), dtype=torch.float32, device=dofs.device),
                    torch.empty(n, dtype=torch.int32, device=dofs.device))
        return (np.empty((n, DOF_WIDTH), np.float32), np.empty((n, RESULT_WIDTH), np.float32),
                np.empty(n, np.int32))

    def minimize_6d(self, rec: int, lig: int, grid: int, params: int, dofs, max_evals: int = 500,
                    stream=None):
        """Device-resident VA13 per pose: (last state (n,6), last result (n,7), evals (n,))."""
        dofs = _check_poses(dofs, DOF_WIDTH, "minimize_6d")
        st, res, nev = self._min_outputs(dofs)
        self._check(self.lib.gba_minimize_6d(self.h, rec, lig, grid, params, _lib.ptr(dofs),
                                             dofs.shape[0], int(max_evals), _lib.ptr(st),
                                             _lib.ptr(res), _lib.ptr(nev), stream))
        return st, res, nev

    def minimize_6d_plain(self, rec: int, lig: int, grid: int, params: int, dofs,
                          max_evals: int = 500, item_size: int = 0, stream=None):
        """Host VA13; per evaluation round one launch per work item of `item_size`
        active poses (0: one launch per round).  Host arrays only."""
        dofs = np.ascontiguousarray(dofs, dtype=np.float32)
        st, res, nev = self._min_outputs(dofs)
        self._check(self.lib.gba_minimize_6d_plain(self.h, rec, lig, grid, params, _lib.ptr(dofs),
                                                   dofs.shape[0], int(max_evals), int(item_size),
                                                   _lib.ptr(st), _lib.ptr(res), _lib.ptr(nev),
                                                   stream))
        return st, res, nev

    def _modes_min(self, fn, rec, lig, grid_rec, grid_lig, params, dofs, max_evals, stream,
                   item_size=None):
        n = dofs.shape[0]
        if _is_torch(dofs):
            import torch
            st = torch.empty((n, DOF_MODES_WIDTH), dtype=torch.float32, device=dofs.device)
            res = torch.empty((n, RESULT_MODES_WIDTH), dtype=torch.float32, device=dofs.device)
            nev = torch.empty(n, dtype=torch.int32, device=dofs.device)
        else:
            st = np.empty((n, DOF_MODES_WIDTH), np.float32)
            res = np.empty((n, RESULT_MODES_WIDTH), np.float32)
            nev = np.empty(n, np.int32)
        extra = () if item_size is None else (int(item_size),)
        self._check(fn(self.h, rec, lig, grid_rec, grid_lig, params, _lib.ptr(dofs), n, int(max_evals),
                       *extra, _lib.ptr(st), _lib.ptr(res), _lib.ptr(nev), stream))
        return st, res, nev

    def minimize_6d_modes(self, rec, lig, grid_rec, grid_lig, params, dofs, max_evals=500,
                          stream=None):
        """Device VA13 over (ang, pos, modesRec, modesLig): (state (n,26), result (n,27), evals)."""
        dofs = _check_poses(dofs, DOF_MODES_WIDTH, "minimize_6d_modes")
        return self._modes_min(self.lib.gba_minimize_6d_modes, rec, lig, grid_rec, grid_lig, params,
                               dofs, max_evals, stream)

    def minimize_6d_modes_plain(self, rec, lig, grid_rec, grid_lig, params, dofs, max_evals=500,
                                item_size=0, stream=None):
        """Host VA13, one round of work items of item_size poses (0: one
        launch per round) per evaluation; host arrays only."""
        dofs = np.ascontiguousarray(dofs, dtype=np.float32)
        return self._modes_min(self.lib.gba_minimize_6d_modes_plain, rec, lig, grid_rec, grid_lig,
                               params, dofs, max_evals, stream, item_size=item_size)

    def _jobs(self, pairs, with_state: bool):
        """pairs: list of (rec, lig, grid, params, dofs) -> (ctypes array, outputs)."""
        jobs = (_lib.PairJobC * len(pairs))()
        outs = []
        for k, (rec, lig, grid, params, dofs) in enumerate(pairs):
            dofs = _check_poses(dofs, DOF_WIDTH, "batch")
            st, res, nev = self._min_outputs(dofs)
            j = jobs[k]
            j.rec, j.lig, j.grid, j.params = rec, lig, grid, params
            j.start, j.n = _lib.ptr(dofs), dofs.shape[0]
            j.out_state = _lib.ptr(st) if with_state else None
            j.out_result = _lib.ptr(res)
            j.out_nevals = _lib.ptr(nev) if with_state else None
            outs.append((dofs, st, res, nev))
        return jobs, outs

    def batch_energy_6d(self, pairs, stream=None):
        """One launch over the poses of many pairs; returns a list of (n_k, 7) results."""
        jobs, outs = self._jobs(pairs, with_state=False)
        self._check(self.lib.gba_batch_energy_6d(self.h, jobs, len(pairs), stream))
        return [o[2] for o in outs]

    def batch_minimize_6d(self, pairs, max_evals: int = 500, stream=None, done_ns: bool = False):
        """One persistent launch minimizing the poses of many pairs; list of (state, result, evals)
        per pair, plus (done_ns) each pose's completion time in ns from the launch's start."""
        jobs, outs = self._jobs(pairs, with_state=True)
        done = []
        if done_ns:
            for k, o in enumerate(outs):
                d = np.zeros(o[0].shape[0], np.uint64)
                jobs[k].out_done_ns = _lib.ptr(d)
                done.append(d)
        self._check(self.lib.gba_batch_minimize_6d(self.h, jobs, len(pairs), int(max_evals), stream))
        if done_ns:
            return [(o[1], o[2], o[3], d) for o, d in zip(outs, done)]
        return [(o[1], o[2], o[3]) for o in outs]

    def set_minimize_team(self, warps_per_pose: int):
        """Warps per pose of the device minimizer (0 = chosen from the job size)."""
        self._check(self.lib.gba_set_minimize_team(self.h, int(warps_per_pose)))

    def set_deadline(self, milliseconds: int):
        self._check(self.lib.gba_set_deadline(self.h, int(milliseconds)))

    def autotune(self, rec: int, lig: int, grid: int, params: int, sample, max_evals: int = 50,
                 cache_path: str | None = None) -> dict:
        """Times launch shapes on `sample` poses; returns the chosen shapes."""
        sample = _check_poses(sample, DOF_WIDTH, "autotune")
        r = _lib.TuneResultC()
        self._check(self.lib.gba_autotune(self.h, rec, lig, grid, params, _lib.ptr(sample),
                                          sample.shape[0], int(max_evals),
                                          cache_path.encode() if cache_path else None, C.byref(r)))
        return {k: getattr(r, k) for k, _ in _lib.TuneResultC._fields_}

    def set_pair_shape(self, rec: int, lig: int, grid: int, params: int, energy_threads: int = 256,
                       energy_blocks_per_sm: int = 64, minimize_threads: int = 128, minimize_chunk: int = 1,
                       minimize_team: int = 1):
        """Sets the pair's launch shapes without timing (as gba_autotune keeps them)."""
        r = _lib.TuneResultC(energy_threads=energy_threads, energy_blocks_per_sm=energy_blocks_per_sm,
                             minimize_threads=minimize_threads, minimize_chunk=minimize_chunk,
                             minimize_team=minimize_team)
        self._check(self.lib.gba_set_pair_shape(self.h, rec, lig, grid, params, C.byref(r)))

    def grid_octets(self, grid: int, enable: bool = True):
        """Adds / drops the duplicated-octet copy of a grid (8x memory, same results)."""
        self._check(self.lib.gba_grid_octets(self.h, grid, int(bool(enable))))

    def set_pose_order(self, enable: bool):
        """Visit large batches grouped by pose translation (default on)."""
        self._check(self.lib.gba_set_pose_order(self.h, int(bool(enable))))

    def set_kernel_options(self, flags: int):
        """GBA_KOPT_* flags: 1 = computed plateau ratio, 2 = 8 lanes per grid
        lookup, 4 = four-block instantiation, 8 = list entries carrying the
        receptor type, 16 = the reference CPU path's summation order (bit for
        bit the reference's results, slower); the default is 15."""
        self._check(self.lib.gba_set_kernel_options(self.h, int(flags)))

    def set_host_sincos(self, max_abs: float = 4096.0):
        """Take each angle's sin/cos from this process's C library (sinf/cosf),
        tabulated on the device for |angle| in [2^-12, max_abs); 0 turns it off."""
        self._check(self.lib.gba_set_host_sincos(self.h, float(max_abs)))

    def kernel_timing(self, enable: bool):
        """Record CUDA events around every fused rigid energy kernel launch."""
        self._check(self.lib.gba_kernel_timing(self.h, int(bool(enable))))

    def kernel_time(self, reset: bool = True) -> tuple[float, int]:
        """(summed kernel ms, launches) recorded since the last reset."""
        import ctypes as C
        ms, n = C.c_double(), C.c_uint64()
        self._check(self.lib.gba_kernel_time(self.h, C.byref(ms), C.byref(n), int(bool(reset))))
        return ms.value, n.value

    def census_6d(self, rec: int, lig: int, grid: int, params: int, dofs):
        """Per-pose counts {n_grid, n_grid_charged, n_nl, n_nl_entries} (n, 4) uint32."""
        dofs = _check_poses(dofs, DOF_WIDTH, "census_6d")
        n = dofs.shape[0]
        res = _alloc_like(dofs, (n, RESULT_WIDTH))
        if _is_torch(dofs):
            import torch
            cen = torch.empty((n, 4), dtype=torch.int32, device=dofs.device)
        else:
            cen = np.empty((n, 4), dtype=np.uint32)
        self._check(self.lib.gba_census_6d(self.h, rec, lig, grid, params, _lib.ptr(dofs), n,
                                           _lib.ptr(res), _lib.ptr(cen)))
        return cen, res
