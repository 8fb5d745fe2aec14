"""Krylov solvers and time-stepping drivers on the GPU against the oracle:
the same reference algorithms (minres.hpp, pcg.hpp, schrodinger.hpp) on the
same inputs.  Iterates differ only by rounding, so iteration counts agree to
a few and solutions to a small multiple of the solver tolerance."""
import numpy as np
import pytest

from tests.util import SMALL_MESH, rel_err, structured

pytestmark = pytest.mark.gpu


def test_poisson_small_mesh(semlib, oracle, known):
    p = known["poisson_p"]
    ctx = semlib.Context(p, folder=SMALL_MESH)
    om = oracle.Mesh(p, folder=SMALL_MESH)
    X, Y = om.node_coords()
    f = X * X - Y * Y
    u_ref, (ok_r, it_r, res_r) = om.poisson(om.zeros(), f, om.dof(), known["poisson_tol"])
    u = np.zeros(om.shape)
    ok, it, res = ctx.poisson(u, f, om.dof(), known["poisson_tol"])
    assert ok and ok_r
    assert abs(it - it_r) <= 3
    assert rel_err(om.unmask(u), om.unmask(u_ref)) <= 1e-8
    # the true residual of the GPU solution meets the reference's criterion
    b = om.gproj(f)
    r = b - om.apply_laplace(u)
    assert np.sqrt(om.dot(r, r)) <= 10 * known["poisson_tol"] * np.sqrt(om.dot(b, b))


def test_poisson_device_pointers_and_zero_guess(semlib, oracle):
    co, el = structured(8, jitter=0.15, seed=0)
    ctx = semlib.Context(4, coords=co, elements=el)
    om = oracle.Mesh(4, coords=co, elements=el)
    X, Y = om.node_coords()
    f = 2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
    b = ctx.gproj(ctx.to_device(f))
    x = ctx.zeros()
    ok, it, res = ctx.pcg_laplace(x, b, 10 * om.dof(), 1e-12, x_is_zero=True)
    u_ref, (ok_r, it_r, _) = om.poisson(om.zeros(), f, 10 * om.dof(), 1e-12)
    assert ok and abs(it - it_r) <= 3
    assert rel_err(om.unmask(x.cpu().numpy()), om.unmask(u_ref)) <= 1e-9


def test_helmholtz_small_mesh(semlib, oracle, known):
    p = known["helmholtz_p"]
    ctx = semlib.Context(p, folder=SMALL_MESH)
    om = oracle.Mesh(p, folder=SMALL_MESH)
    X, Y = om.node_coords()
    f = X * X - Y * Y
    c = np.full(om.shape, known["helmholtz_c"])
    u_ref, (ok_r, it_r, res_r) = om.helmholtz(om.zeros(), c, f, 10 * om.dof(), known["helmholtz_tol"])
    u = np.zeros(om.shape)
    ok, it, res = ctx.helmholtz(u, c, f, 10 * om.dof(), known["helmholtz_tol"])
    assert ok and ok_r
    assert abs(it - it_r) <= max(5, it_r // 50)
    assert rel_err(om.unmask(u), om.unmask(u_ref)) <= 1e-7


def test_minres_nonzero_guess_and_maxit(semlib, oracle):
    ctx = semlib.Context(3, folder=SMALL_MESH)
    om = oracle.Mesh(3, folder=SMALL_MESH)
    rng = np.random.default_rng(3)
    c = np.full(om.shape, -20.0)
    b = om.mask(om.global_sum(rng.standard_normal(om.shape)))
    x0 = rng.standard_normal(om.shape)
    import ctypes as C
    # maxit = 5: not converged, n_iter = maxit + 1 (minres.hpp:46,105)
    x = ctx.to_device(x0)
    ok, it, res = ctx.minres_helmholtz(ctx.to_device(c), x, ctx.to_device(b), 5, 1e-12)
    assert not ok and it == 6
    x_ref, (ok_r, it_r, res_r) = oracle.krylov("minres", lambda v: om.apply_helmholtz(c, v.reshape(om.shape)).ravel(),
                                               b.ravel(), x0.ravel(), 5, 1e-12,
                                               dot=lambda a, bb: om.dot(a.reshape(om.shape), bb.reshape(om.shape)))
    assert it_r == 6 and abs(res - res_r) <= 1e-10 * res_r
    assert rel_err(x.cpu().numpy().ravel(), x_ref) <= 1e-11


def _schro_case(om, kind):
    X, Y = om.node_coords()
    if kind == "ref":  # tests/schrodinger.cpp
        return np.sin(np.pi * X) * np.sin(np.pi * Y), om.zeros(), om.zeros()
    from schrodingersem_gb300.meshgen import gaussian_packet
    re, im = gaussian_packet(X, Y, (-0.3, 0.1), 0.4, (3.0, 1.0))
    return re, im, 0.5 * (X * X + Y * Y)


@pytest.mark.parametrize("method", ["bdf2", "dirk4s3", "dirk4s5"])
@pytest.mark.parametrize("kind", ["ref", "packet"])
def test_schrodinger_drivers(semlib, oracle, known, method, kind):
    if kind == "ref":
        p = known["schro_p"]
        ctx = semlib.Context(p, folder=SMALL_MESH)
        om = oracle.Mesh(p, folder=SMALL_MESH)
        T, steps, tol = known["schro_T"], known["schro_steps"], known["schro_tol"]
    else:
        co, el = structured(6, box=(-2, 2, -2, 2), jitter=0.1, seed=1)
        ctx = semlib.Context(5, coords=co, elements=el)
        om = oracle.Mesh(5, coords=co, elements=el)
        T, steps, tol = 0.05, 5, 1e-10
    re, im, V = _schro_case(om, kind)
    dt = T / steps
    rec_r = []
    pr, pi, ok_r = om.schrodinger(method, re, im, V, T, dt, 20 * om.dof(), tol, record=rec_r)
    gr, gi = re.copy(), im.copy()
    rec = []
    ok = ctx.schrodinger(method, gr, gi, V, T, dt, 20 * om.dof(), tol, record=rec)
    assert ok and ok_r
    assert len(rec) == len(rec_r) == steps
    for (s1, it1), (s2, it2) in zip(rec, rec_r):
        assert s1 == s2 and all(abs(a - b) <= 3 for a, b in zip(it1, it2))
    # minres.hpp:92 stops at phibar < tol*|r0| + tol, so with |b| << 1 a stage
    # is accurate to about tol/|b|: judge both runs against a tight solve
    tr, ti, _ = om.schrodinger(method, re, im, V, T, dt, 20 * om.dof(), 1e-14)
    e_gpu = max(rel_err(gr, tr), rel_err(gi, ti))
    e_ref = max(rel_err(pr, tr), rel_err(pi, ti))
    assert e_gpu <= 3 * e_ref + 1e-11, (e_gpu, e_ref)
    assert max(rel_err(gr, pr), rel_err(gi, pi)) <= 4 * e_ref + 1e-11


def test_callback_stops_and_state_visible(semlib, oracle, known):
    ctx = semlib.Context(3, folder=SMALL_MESH)
    om = oracle.Mesh(3, folder=SMALL_MESH)
    re, im, V = _schro_case(om, "ref")
    gr, gi = re.copy(), im.copy()
    rec = []
    ok = ctx.schrodinger("dirk4s3", gr, gi, V, 1.0, 0.001, 20 * om.dof(), 1e-8, n_steps=3, record=rec)
    assert ok and [s for s, _ in rec] == [1, 2, 3]
    pr, pi, _ = om.schrodinger("dirk4s3", re, im, V, 1.0, 0.001, 20 * om.dof(), 1e-8, n_steps=3)
    assert rel_err(gr, pr) <= 1e-6


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_adaptive_dirk4s5_replays_fixed_step_reference(semlib, oracle, prec):
    """adaptive SDIRK4-5: every accepted step's embedded estimate is within
    the tolerance, the steps land on T, and replaying the accepted dt
    sequence through the oracle's fixed-step 5-stage driver reproduces the
    state"""
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.meshgen import gaussian_packet
    co, el = structured(4, box=(-3, 3, -3, 3), jitter=0.1, seed=5)
    p = 5
    ctx = semlib.Context(p, coords=co, elements=el)
    om = oracle.Mesh(p, coords=co, elements=el)
    X, Y = om.node_coords()
    re, im = gaussian_packet(X, Y, (-0.5, 0.2), 0.7, (2.0, 1.0))
    V = X * X + Y * Y
    if prec == "mixed":
        ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
        ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
        ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
        ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    T, tol, err_tol = 0.06, 1e-12, 1e-6
    a, b = re.copy(), im.copy()
    ok, dts, nrej = ctx.schrodinger_adaptive(a, b, V, T, 0.02, 100000, tol, err_tol)
    assert ok and len(dts) >= 2
    assert abs(dts.sum() - T) < 1e-12
    assert ctx.stats().last_error_estimate <= err_tol
    # the controller moved away from the 0.02 trial step
    assert nrej > 0 or abs(dts[-2] - 0.02) > 1e-12
    r, i = re.copy(), im.copy()
    for d in dts:
        r, i, okk = om.schrodinger("dirk4s5", r, i, V, 0.5 * d, d, 100000, 1e-13)
        assert okk
    assert max(rel_err(a, r), rel_err(b, i)) < 1e-8
