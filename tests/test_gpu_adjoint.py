"""The autograd adjoint of the pairwise path against FP64 central finite
differences (step 1e-4, pair set frozen at the unperturbed pose so the
difference quotient sees one smooth function; the five-point stencil
(f(-2h) - 8 f(-h) + 8 f(h) - f(2h)) / 12h, because in a clash the three-point
quotient's own truncation error reaches 4e-3 at config 3's size while the
five-point one stays near 2e-5 of the FP64 analytic gradient) and against the analytic
forces / torques reduced the reference's way (TorqueMat), plus the grid path
whose backward is the reference's own -Result.

Every check runs on a small pair (150/60 beads) and on config 3's system:
config 1's 2000/700-bead pair with a 200-pose subset of its 10,000 poses,
as the finite-difference check of that configuration asks.

Tolerance: |adjoint - reference| <= 1e-4 * max(|reference|, 1e-3 * max over
the batch) per component (the floor covers components that cancel to ~0)."""
import numpy as np
import pytest

from test_gpu_rigid import upload

pytestmark = pytest.mark.gpu

H = 1e-4


def five_point(f):
    """Central difference of step H with the five-point stencil; f(m) is the
    function at the base point moved by m * H."""
    return (f(-2) - 8 * f(-1) + 8 * f(1) - f(2)) / (12 * H)


def scaled_err(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    floor = 1e-3 * np.max(np.abs(ref), axis=0, keepdims=True) + 1e-300
    return np.abs(got - ref) / np.maximum(np.abs(ref), floor)


@pytest.fixture(scope="module", params=["small", "config3"])
def adj_case(request, pkg, oracle):
    import torch
    from gbattract.autograd import PairwiseSystem
    from gbattract.context import GbaContext
    rng = np.random.default_rng(31)
    if request.param == "small":
        wl = pkg.synth.make_pair(3, 150, 60, 200, (19.0, 27.0), seed=3131)
    else:
        wl = pkg.synth.make_config(3)
        wl.dofs = np.ascontiguousarray(wl.dofs[:200])
    T = 32
    r0 = rng.uniform(3.0, 5.0, (T, T)).astype(np.float32)
    eps = rng.uniform(0.1, 10.0, (T, T)).astype(np.float32)
    ipon = np.ones((T, T), np.int32)
    ipon[rng.random((T, T)) < 0.2] = 0          # exercise the emin branch too
    q_lig = (wl.lig.charge + rng.normal(0, 0.1, wl.lig.n)).astype(np.float32)
    q_rec = (wl.rec.charge + rng.normal(0, 0.1, wl.rec.n)).astype(np.float32)
    ctx = GbaContext(0)
    rec, lig, par = ctx.upload_protein(wl.rec), ctx.upload_protein(wl.lig), ctx.upload_params(wl.params)
    # neighbour-list candidates only (the pairwise path reads no potentials):
    # the device-built grid, bit-identical to the oracle's
    ids = (rec, lig, ctx.build_grid(rec, par, pkg.GridOptions()), par)
    sysm = PairwiseSystem(ctx=ctx, rec=ids[0], lig=ids[1], grid=ids[2],
                          ipon=torch.from_numpy(ipon).cuda(), ffelec=wl.params.ffelec)
    yield dict(wl=wl, r0=r0, eps=eps, ipon=ipon, q_lig=q_lig, q_rec=q_rec, ctx=ctx,
               ids=ids, sysm=sysm)
    ctx.close()


def ref_energy(oracle, c, dofs, q_lig=None, q_rec=None, r0=None, eps=None, ref=None, grad=False):
    wl = c["wl"]
    return oracle.pairwise_energy_f64(
        wl.rec, wl.lig, c["q_rec"] if q_rec is None else q_rec, c["q_lig"] if q_lig is None else q_lig,
        c["r0"] if r0 is None else r0, c["eps"] if eps is None else eps, c["ipon"],
        wl.params.dielec, wl.params.ffelec, 10.0, dofs, ref_dofs6=ref, grad=grad)


def run_adjoint(c):
    import torch
    from gbattract.autograd import PairwiseEnergy
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda().requires_grad_(True)
    d, ql, qr, r0, eps = (t(c["wl"].dofs), t(c["q_lig"]), t(c["q_rec"]), t(c["r0"]), t(c["eps"]))
    E = PairwiseEnergy.apply(d, ql, qr, r0, eps, c["sysm"])
    E.sum().backward()
    return (E.detach().cpu().numpy(), d.grad.cpu().numpy(), ql.grad.cpu().numpy(),
            qr.grad.cpu().numpy(), r0.grad.cpu().numpy(), eps.grad.cpu().numpy())


def test_forward_matches_fp64(oracle, adj_case):
    E, *_ = run_adjoint(adj_case)
    ref = ref_energy(oracle, adj_case, adj_case["wl"].dofs.astype(np.float64))
    assert float(scaled_err(E[:, None], ref[:, None]).max()) <= 1e-4


def test_dof_gradient_vs_analytic_and_fd(oracle, adj_case):
    _, gd, *_ = run_adjoint(adj_case)
    base = adj_case["wl"].dofs.astype(np.float64)
    _, g_an = ref_energy(oracle, adj_case, base, grad=True)
    assert float(scaled_err(gd, g_an).max()) <= 1e-4
    fd = np.zeros_like(g_an)
    for k in range(6):
        def at(m):
            d = base.copy()
            d[:, k] += m * H
            return ref_energy(oracle, adj_case, d, ref=base)
        fd[:, k] = five_point(at)
    err = scaled_err(gd, fd)
    print(f"dE/dDOF vs FD: max scaled error {err.max():.2e}, median {np.median(err):.2e}")
    assert float(err.max()) <= 1e-4


def test_parameter_gradients_vs_fd(oracle, adj_case):
    _, _, gql, gqr, gr0, geps = run_adjoint(adj_case)
    base = adj_case["wl"].dofs.astype(np.float64)
    rng = np.random.default_rng(5)

    def fd_of(name, idx, arr):
        def at(m):
            a = arr.astype(np.float64).copy()
            a.flat[idx] += m * H
            return ref_energy(oracle, adj_case, base, **{name: a}).sum()
        return five_point(at)

    # type pairs that occur in contacts: largest adjoint magnitudes plus random ones
    cand = list(np.argsort(-np.abs(gr0.ravel()))[:6]) + list(rng.integers(0, gr0.size, 3))
    got, want = [], []
    for idx in cand:
        got += [gr0.flat[idx], geps.flat[idx]]
        want += [fd_of("r0", idx, adj_case["r0"]), fd_of("eps", idx, adj_case["eps"])]
    for idx in list(np.argsort(-np.abs(gql))[:4]) + list(rng.integers(0, gql.size, 2)):
        got.append(gql[idx])
        want.append(fd_of("q_lig", idx, adj_case["q_lig"]))
    for idx in list(np.argsort(-np.abs(gqr))[:4]) + list(rng.integers(0, gqr.size, 2)):
        got.append(gqr[idx])
        want.append(fd_of("q_rec", idx, adj_case["q_rec"]))
    got, want = np.array(got), np.array(want)
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-3 * np.abs(want).max())
    print(f"parameter gradients vs FD: max scaled error {rel.max():.2e}")
    assert float(rel.max()) <= 1e-4


def test_grid_energy_backward_is_minus_result(small_case, pkg):
    import torch
    from gbattract.autograd import GridEnergy
    from gbattract.context import GbaContext
    wl, grid = small_case
    with GbaContext(0) as ctx:
        ids = upload(ctx, wl.rec, wl.lig, grid, wl.params)
        d = torch.from_numpy(wl.dofs).cuda().requires_grad_(True)
        w = torch.linspace(0.5, 1.5, len(wl.dofs), device="cuda")
        E = GridEnergy.apply(d, (ctx, *ids))
        (E * w).sum().backward()
        res = ctx.energy_6d(*ids, wl.dofs)
        assert np.array_equal(E.detach().cpu().numpy(), res[:, 0])
        want = -res[:, 1:7] * w.cpu().numpy()[:, None]
        assert np.allclose(d.grad.cpu().numpy(), want, rtol=1e-6, atol=0)


def test_nearest_first_order_keeps_every_result(adj_case):
    """From 2,048 poses on, the pairwise kernels visit poses nearest the
    receptor centre first; each pose's energy and DOF gradient is its own
    (bit for bit the same as in batches below the threshold, which keep
    submission order), and the summed parameter gradients agree up to FP64
    summation order."""
    import torch
    from gbattract.autograd import PairwiseEnergy
    c = adj_case
    rng = np.random.default_rng(47)
    base = c["wl"].dofs
    dofs = base[rng.integers(0, len(base), 2600)].copy()
    dofs[:, :3] += rng.normal(0, 2.0, (len(dofs), 3)).astype(np.float32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda().requires_grad_(True)

    def run(d_np):
        d, ql, qr, r0, eps = (t(d_np), t(c["q_lig"]), t(c["q_rec"]), t(c["r0"]), t(c["eps"]))
        E = PairwiseEnergy.apply(d, ql, qr, r0, eps, c["sysm"])
        E.sum().backward()
        return [x.detach().cpu().numpy().astype(np.float64) for x in (E, d.grad, ql.grad, qr.grad, r0.grad, eps.grad)]

    whole = run(dofs)
    parts = [run(dofs[k:k + 650]) for k in range(0, len(dofs), 650)]
    assert np.array_equal(whole[0], np.concatenate([p[0] for p in parts]))
    assert np.array_equal(whole[1], np.concatenate([p[1] for p in parts]))
    for i in range(2, 6):
        summed = np.sum([p[i] for p in parts], axis=0)
        scale = np.max(np.abs(summed)) + 1e-30
        assert np.max(np.abs(whole[i] - summed)) <= 1e-5 * scale
