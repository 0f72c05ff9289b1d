"""torch.autograd Functions over the batched pose energy.

PairwiseEnergy  forward: exact ATTRACT pair energy per pose (pairs within the
                cutoff, no grid), one fused launch; backward: the hand-written
                adjoint kernel (gba_pairwise_6d with an upstream gradient),
                which recomputes the transformed coordinates and returns
                dE/dDOF, dE/d(ligand / receptor charges) and dE/d(r0, eps) per
                type pair -- the parameters of a scoring-function refit.
GridEnergy      forward: the reference-equivalent grid + NL energy
                (gba_energy_6d); backward: -Result, i.e. the reference's own
                analytic forces and Euler torques (src/apps/em/meta.h:114-121).

Poses are (n, 6) float32 CUDA tensors in DOF_6D order (pos xyz, ang xyz);
gradients come back in the same layout.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib
from .model import DIELEC_VARIABLE, FELEC, POTSHAPE_8_6


class PairwiseParamsC(C.Structure):
    _fields_ = [("num_types", C.c_uint32), ("r0", C.c_void_p), ("eps", C.c_void_p),
                ("ipon", C.c_void_p), ("q_lig", C.c_void_p), ("q_rec", C.c_void_p),
                ("potshape", C.c_int), ("dielec", C.c_int), ("ffelec", C.c_float),
                ("cutoff", C.c_float)]


@dataclass
class PairwiseSystem:
    """Device-side handles of one receptor-ligand pair for the pairwise path."""
    ctx: object           # GbaContext
    rec: int
    lig: int
    grid: int             # supplies the neighbour lists
    ipon: torch.Tensor    # (T, T) int32, CUDA
    dielec: int = DIELEC_VARIABLE
    ffelec: float = float(torch.tensor(FELEC / 15.0, dtype=torch.float32))
    cutoff: float = 10.0


def _call(sysm: PairwiseSystem, dofs, q_lig, q_rec, r0, eps, E=None, gE=None, gd=None, gql=None,
          gqr=None, gr0=None, geps=None):
    lib = _lib.load()
    if not hasattr(lib.gba_pairwise_6d, "_typed"):
        P, U32, SZ = C.c_void_p, C.c_uint32, C.c_size_t
        lib.gba_pairwise_6d.argtypes = [P, U32, U32, U32, C.POINTER(PairwiseParamsC), P, SZ, P, P,
                                        P, P, P, P, P, P]
        lib.gba_pairwise_6d.restype = C.c_int
        lib.gba_pairwise_6d._typed = True
    pp = PairwiseParamsC()
    pp.num_types = r0.shape[0]
    pp.r0, pp.eps, pp.ipon = r0.data_ptr(), eps.data_ptr(), sysm.ipon.data_ptr()
    pp.q_lig, pp.q_rec = q_lig.data_ptr(), q_rec.data_ptr()
    pp.potshape, pp.dielec = POTSHAPE_8_6, sysm.dielec
    pp.ffelec, pp.cutoff = sysm.ffelec, sysm.cutoff
    p = lambda t: None if t is None else t.data_ptr()
    stream = torch.cuda.current_stream(dofs.device).cuda_stream
    rc = lib.gba_pairwise_6d(sysm.ctx.h, sysm.rec, sysm.lig, sysm.grid, C.byref(pp), p(dofs),
                             dofs.shape[0], p(E), p(gE), p(gd), p(gql), p(gqr), p(gr0), p(geps),
                             stream)
    _lib.check(sysm.ctx.h, rc)


def _f32(t):
    return t.detach().to(torch.float32).contiguous()


class PairwiseEnergy(torch.autograd.Function):
    """E = PairwiseEnergy.apply(dofs, q_lig, q_rec, r0, eps, system) -> (n,) float32."""

    @staticmethod
    def forward(ctx, dofs, q_lig, q_rec, r0, eps, system: PairwiseSystem):
        d, ql, qr, a, b = map(_f32, (dofs, q_lig, q_rec, r0, eps))
        E = torch.empty(d.shape[0], dtype=torch.float32, device=d.device)
        _call(system, d, ql, qr, a, b, E=E)
        ctx.save_for_backward(d, ql, qr, a, b)
        ctx.system = system
        return E

    @staticmethod
    def backward(ctx, gE):
        d, ql, qr, a, b = ctx.saved_tensors
        gE = gE.detach().to(torch.float32).contiguous()
        dev = d.device
        gd = torch.empty_like(d)
        gql = torch.zeros(ql.shape, dtype=torch.float64, device=dev)
        gqr = torch.zeros(qr.shape, dtype=torch.float64, device=dev)
        gr0 = torch.zeros(a.shape, dtype=torch.float64, device=dev)
        geps = torch.zeros(b.shape, dtype=torch.float64, device=dev)
        _call(ctx.system, d, ql, qr, a, b, gE=gE, gd=gd, gql=gql, gqr=gqr, gr0=gr0, geps=geps)
        return gd, gql.to(torch.float32), gqr.to(torch.float32), gr0.to(torch.float32), \
            geps.to(torch.float32), None


class GridEnergy(torch.autograd.Function):
    """E = GridEnergy.apply(dofs, (ctx, rec, lig, grid, params)) -> (n,) float32."""

    @staticmethod
    def forward(ctx, dofs, handles):
        gctx, rec, lig, grid, params = handles
        d = _f32(dofs)
        res = gctx.energy_6d(rec, lig, grid, params, d,
                             stream=torch.cuda.current_stream(d.device).cuda_stream)
        ctx.save_for_backward(res)
        return res[:, 0].clone()

    @staticmethod
    def backward(ctx, gE):
        (res,) = ctx.saved_tensors
        g = -res[:, 1:7] * gE.to(torch.float32)[:, None]      # -(force, torque) = dE/d(pos, ang)
        return g, None
