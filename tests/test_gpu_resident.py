"""The on-chip resident FP32 inner solve (SEM_OPT_RESIDENT, default on).

Mixed-precision stage solves with the element preconditioner keep the inner
Krylov vectors in shared memory and registers when each SM's share of the
mesh fits, exchanging only element-ring copies through global memory.  The
FP64 refinement around it is unchanged, so against the staged kernel
(SEM_OPT_RESIDENT = 0) and the plain FP64 solver the solutions must agree to
the solver tolerance's accuracy, meet the reference's residual criterion on
the true FP64 residual (include/minres.hpp:92), be deterministic (the grid
sums are formed in one fixed order), and fall back to the staged kernel when
a block's share does not fit."""
import ctypes as C

import numpy as np
import pytest

from tests.util import SMALL_MESH, rel_err, structured

pytestmark = pytest.mark.gpu

SEM_ERR_DEVICE_WAIT = 5


def _case(semlib, oracle, n, p, box=8.0, seed=1, folder=None, neumann=False):
    from schrodingersem_gb300.meshgen import gaussian_packet
    if folder:
        ctx = semlib.Context(p, folder=folder, neumann=neumann)
        om = oracle.Mesh(p, folder=folder, neumann=neumann)
    else:
        co, el = structured(n, box=(-box, box, -box, box), jitter=0.1, seed=seed)
        ctx = semlib.Context(p, coords=co, elements=el, neumann=neumann)
        om = oracle.Mesh(p, coords=co, elements=el, neumann=neumann)
    X, Y = om.node_coords()
    s = 0.25 * box if not folder else 0.2
    re, im = gaussian_packet(X, Y, (-0.25 * box if not folder else 0.3, 0.1), s, (3.0, -1.0))
    V = 0.5 * (X * X + Y * Y) if not folder else 10 * (X * X + Y * Y)
    return ctx, om, re, im, V


def _stage(ctx, V, re, im, dt=0.005):
    dV = ctx.to_device(V)
    br, bi = ctx.schro_f(dV, ctx.to_device(re), ctx.to_device(im))
    br.mul_(dt)
    bi.mul_(dt)
    return dV, br, bi, dt * 1.0886


def _mixed_fdm(ctx, resident):
    from schrodingersem_gb300 import capi
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_RESIDENT, 1 if resident else 0)


def _true_residual_ok(om, V, alpha, b, x, tol):
    Ax = om.schro_res(V, alpha, x[0], x[1])
    r = np.sqrt(om.dot(b[0] - Ax[0], b[0] - Ax[0]) + om.dot(b[1] - Ax[1], b[1] - Ax[1]))
    bn = np.sqrt(om.dot(b[0], b[0]) + om.dot(b[1], b[1]))
    return r < tol * bn + tol, r / bn


@pytest.mark.parametrize("n,p", [(64, 8), (40, 8), (30, 6), (48, 4), (20, 10), (10, 8)])
def test_resident_matches_staged_and_fp64(semlib, oracle, n, p):
    """several elements per block (64x64 at p = 8 is 27 per SM on 152 SMs),
    one element per block (10x10), every resident degree"""
    ctx, om, re, im, V = _case(semlib, oracle, n, p)
    dV, br, bi, alpha = _stage(ctx, V, re, im)
    tol = 1e-11
    xr, xi = ctx.zeros(), ctx.zeros()
    ok64, _, _ = ctx.minres_schro(dV, alpha, xr, xi, br, bi, 20 * ctx.dof(), tol, x_is_zero=True)
    out = {}
    for resident in (False, True):
        _mixed_fdm(ctx, resident)
        s0 = ctx.stats().resident_launches
        yr, yi = ctx.zeros(), ctx.zeros()
        ok, it, _ = ctx.minres_schro(dV, alpha, yr, yi, br, bi, 20 * ctx.dof(), tol, x_is_zero=True)
        assert ok
        assert ctx.stats().resident_launches - s0 == (1 if resident else 0)
        out[resident] = (it, yr.cpu().numpy(), yi.cpu().numpy())
    print(n, p, "inner iterations staged", out[False][0], "resident", out[True][0])
    # same preconditioned iteration: counts within a few iterations per sweep
    assert abs(out[True][0] - out[False][0]) <= max(6, 0.05 * out[False][0])
    b = (br.cpu().numpy(), bi.cpu().numpy())
    ok_r, rel = _true_residual_ok(om, V, alpha, b, out[True][1:], tol)
    assert ok_r, rel
    ref = (xr.cpu().numpy(), xi.cpu().numpy())
    for k in (0, 1):
        assert rel_err(om.unmask(out[True][k + 1]), om.unmask(ref[k])) < 1e-8
        assert rel_err(om.unmask(out[True][k + 1]), om.unmask(out[False][k + 1])) < 1e-8
    assert ok64


@pytest.mark.parametrize("p,neumann", [(4, False), (6, False), (6, True)])
def test_resident_unstructured_mesh(semlib, oracle, p, neumann):
    """the reference's unstructured sample mesh (corner valences 1 to 6),
    Dirichlet and natural (Neumann) boundaries"""
    ctx, om, re, im, V = _case(semlib, oracle, 0, p, folder=SMALL_MESH, neumann=neumann)
    dV, br, bi, alpha = _stage(ctx, V, re, im)
    tol = 1e-11
    xr, xi = ctx.zeros(), ctx.zeros()
    assert ctx.minres_schro(dV, alpha, xr, xi, br, bi, 20 * ctx.dof(), tol, x_is_zero=True)[0]
    _mixed_fdm(ctx, True)
    s0 = ctx.stats().resident_launches
    yr, yi = ctx.zeros(), ctx.zeros()
    assert ctx.minres_schro(dV, alpha, yr, yi, br, bi, 20 * ctx.dof(), tol, x_is_zero=True)[0]
    assert ctx.stats().resident_launches == s0 + 1
    y = (yr.cpu().numpy(), yi.cpu().numpy())
    ok_r, rel = _true_residual_ok(om, V, alpha, (br.cpu().numpy(), bi.cpu().numpy()), y, tol)
    assert ok_r, rel
    assert rel_err(om.unmask(y[0]), om.unmask(xr.cpu().numpy())) < 1e-8
    assert rel_err(om.unmask(y[1]), om.unmask(xi.cpu().numpy())) < 1e-8


def test_resident_deterministic_and_warm_start(semlib, oracle):
    """repeated solves give the same bits; a warm start (x_is_zero = 0)
    converges from the given guess to the reference's criterion"""
    ctx, om, re, im, V = _case(semlib, oracle, 32, 8)
    dV, br, bi, alpha = _stage(ctx, V, re, im)
    _mixed_fdm(ctx, True)
    res = []
    for _ in range(3):
        yr, yi = ctx.zeros(), ctx.zeros()
        ok, it, _ = ctx.minres_schro(dV, alpha, yr, yi, br, bi, 20 * ctx.dof(), 1e-10, x_is_zero=True)
        assert ok
        res.append((it, yr.clone(), yi.clone()))
    for it, yr, yi in res[1:]:
        assert it == res[0][0]
        assert bool((yr == res[0][1]).all()) and bool((yi == res[0][2]).all())
    # warm start (x_is_zero = 0) from the solution perturbed by 1e-3: the
    # true residual meets the reference's test relative to the initial one
    gr, gi = res[0][1] * (1 + 1e-3), res[0][2] * (1 - 1e-3)
    b = (br.cpu().numpy(), bi.cpu().numpy())
    A0 = om.schro_res(V, alpha, gr.cpu().numpy(), gi.cpu().numpy())
    r0 = np.sqrt(om.dot(b[0] - A0[0], b[0] - A0[0]) + om.dot(b[1] - A0[1], b[1] - A0[1]))
    ok, it_w, _ = ctx.minres_schro(dV, alpha, gr, gi, br, bi, 20 * ctx.dof(), 1e-10, x_is_zero=False)
    assert ok
    Ax = om.schro_res(V, alpha, gr.cpu().numpy(), gi.cpu().numpy())
    r = np.sqrt(om.dot(b[0] - Ax[0], b[0] - Ax[0]) + om.dot(b[1] - Ax[1], b[1] - Ax[1]))
    assert r < 1e-10 * r0 + 1e-10, (r, r0)


def test_resident_falls_back_when_share_does_not_fit(semlib, oracle):
    """128x128 elements at p = 8 is 108 elements per SM: above the on-chip
    capacity, so the staged kernel runs (and still converges); odd degrees
    (p = 5) have no resident kernel"""
    for n, p in ((128, 8), (12, 5)):
        ctx, om, re, im, V = _case(semlib, oracle, n, p)
        dV, br, bi, alpha = _stage(ctx, V, re, im)
        _mixed_fdm(ctx, True)
        s0 = ctx.stats()
        yr, yi = ctx.zeros(), ctx.zeros()
        ok, it, _ = ctx.minres_schro(dV, alpha, yr, yi, br, bi, 20 * ctx.dof(), 1e-10, x_is_zero=True)
        s1 = ctx.stats()
        assert ok
        assert s1.resident_launches == s0.resident_launches
        assert s1.solver_launches == s0.solver_launches + 1


def test_resident_wait_limit_expires_and_context_recovers(semlib, oracle):
    """a 1 ns wait limit makes the resident all-reduce's bounded poll give
    up: SEM_ERR_DEVICE_WAIT, no hang; the same context then solves to the
    bits of an undisturbed solve"""
    import torch

    from schrodingersem_gb300 import capi
    ctx, om, re, im, V = _case(semlib, oracle, 24, 8)
    dV, br, bi, alpha = _stage(ctx, V, re, im)
    _mixed_fdm(ctx, True)
    L = capi.load()
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def solve():
        xr, xi = ctx.zeros(), ctx.zeros()
        r = capi.SemSolverResults()
        st = L.sem_minres_schro(ctx._h, p(dV), alpha, p(xr), p(xi), p(br), p(bi), 20 * ctx.dof(), 1e-10, 1,
                                C.byref(r))
        return st, r, xr, xi

    st0, r0, x0r, x0i = solve()
    assert st0 == 0 and r0.success
    ctx.set_option(capi.OPT_WAIT_TIMEOUT_MS, 1e-6)
    st, _, _, _ = solve()
    torch.cuda.synchronize()
    assert st == SEM_ERR_DEVICE_WAIT, st
    ctx.set_option(capi.OPT_WAIT_TIMEOUT_MS, 2000.0)
    st1, r1, x1r, x1i = solve()
    assert st1 == 0 and r1.success and r1.n_iter == r0.n_iter
    assert torch.equal(x1r, x0r) and torch.equal(x1i, x0i)


@pytest.mark.parametrize("method", ["dirk4s3", "bdf2"])
def test_resident_driver_matches_fp64(semlib, oracle, method):
    """whole time steps with the extrapolated stage guess, resident inner
    solves, against the plain FP64 driver"""
    from schrodingersem_gb300 import capi
    ctx, om, re, im, V = _case(semlib, oracle, 24, 8, box=6.0)
    T, steps, tol = 0.04, 4, 1e-10
    a_re, a_im = re.copy(), im.copy()
    assert ctx.schrodinger(method, a_re, a_im, V, T, T / steps, 20 * ctx.dof(), tol)
    _mixed_fdm(ctx, True)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
    s0 = ctx.stats().resident_launches
    b_re, b_im = re.copy(), im.copy()
    assert ctx.schrodinger(method, b_re, b_im, V, T, T / steps, 20 * ctx.dof(), tol)
    assert ctx.stats().resident_launches > s0
    assert max(rel_err(b_re, a_re), rel_err(b_im, a_im)) < 1e-8
