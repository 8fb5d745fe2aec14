"""Projection stage guess (SEM_OPT_PROJECT): the residual-minimising
combination of the last K stage solutions (Fischer's method for successive
right-hand sides).  The stage solve still runs to the same tolerance on the
true FP64 residual, so the trajectory must match the plain FP64 driver to the
metric's 1e-8; the guess must cut the iterations against the extrapolated
guess once the basis has filled, report a residual ratio below 1, reset
when the step size changes, and reject a bad basis size."""
import numpy as np
import pytest

from tests.util import rel_err, structured

pytestmark = pytest.mark.gpu


def _case(semlib, n=24, p=8):
    from schrodingersem_gb300.meshgen import gaussian_packet
    co, el = structured(n, box=(-6.0, 6.0, -6.0, 6.0), jitter=0.1, seed=5)
    ctx = semlib.Context(p, coords=co, elements=el)
    X, Y = ctx.node_coords()
    re, im = gaussian_packet(X, Y, (-1.5, 0.0), 1.0, (3.0, 0.5))
    return ctx, re, im, X * X + Y * Y


def _mixed(ctx, K, guess=1):
    from schrodingersem_gb300 import capi
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    ctx.set_option(capi.OPT_STAGE_GUESS, guess)
    ctx.set_option(capi.OPT_PROJECT, K)


@pytest.mark.parametrize("method", ["dirk4s3", "dirk4s5"])
def test_projection_matches_fp64_and_cuts_iterations(semlib, method):
    ctx, re, im, V = _case(semlib)
    T, steps, tol = 0.08, 8, 1e-10
    a_re, a_im = re.copy(), im.copy()
    assert ctx.schrodinger(method, a_re, a_im, V, T, T / steps, 20 * ctx.dof(), tol)
    its = {}
    for K in (0, 8):
        _mixed(ctx, K)
        b_re, b_im = re.copy(), im.copy()
        rec = []
        s0 = ctx.stats()
        assert ctx.schrodinger(method, b_re, b_im, V, T, T / steps, 20 * ctx.dof(), tol, record=rec)
        s1 = ctx.stats()
        assert max(rel_err(b_re, a_re), rel_err(b_im, a_im)) < 1e-8
        its[K] = s1.krylov_iterations - s0.krylov_iterations
        if K:
            n = s1.projected_guesses - s0.projected_guesses
            stages = 3 if method == "dirk4s3" else 5
            assert n == steps * stages - 1  # every stage but the very first
            assert 0 < (s1.projection_ratio_sum - s0.projection_ratio_sum) / n < 1
            assert s1.last_projection_ratio < 1e-2
    print(method, "inner iterations extrapolated", its[0], "projected", its[8])
    assert its[8] < 0.85 * its[0]


def test_projection_resets_on_new_step_size_and_with_learned_mode(semlib):
    """a new dt starts a new basis (the operator changed); the learned mode
    without a network falls back to the projection"""
    from schrodingersem_gb300 import capi
    ctx, re, im, V = _case(semlib, n=12, p=6)
    tol = 1e-10
    _mixed(ctx, 6, guess=capi.GUESS_LEARNED)
    a_re, a_im = re.copy(), im.copy()
    assert ctx.schrodinger("dirk4s3", a_re, a_im, V, 0.03, 0.01, 20 * ctx.dof(), tol)
    s0 = ctx.stats()
    assert ctx.schrodinger("dirk4s3", a_re, a_im, V, 0.04, 0.02, 20 * ctx.dof(), tol)
    s1 = ctx.stats()
    # the first stage after the change starts from zero: 2 steps x 3 stages - 1
    assert s1.projected_guesses - s0.projected_guesses == 5
    ref_re, ref_im = re.copy(), im.copy()
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_FP64)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_ZERO)
    assert ctx.schrodinger("dirk4s3", ref_re, ref_im, V, 0.03, 0.01, 20 * ctx.dof(), tol)
    assert ctx.schrodinger("dirk4s3", ref_re, ref_im, V, 0.04, 0.02, 20 * ctx.dof(), tol)
    assert max(rel_err(a_re, ref_re), rel_err(a_im, ref_im)) < 1e-8


def test_projection_option_range(semlib):
    from schrodingersem_gb300 import capi
    ctx, _, _, _ = _case(semlib, n=4, p=4)
    for bad in (-1, 25, 2.5):
        with pytest.raises(capi.SemError):
            ctx.set_option(capi.OPT_PROJECT, bad)
    ctx.set_option(capi.OPT_PROJECT, 24)
    ctx.set_option(capi.OPT_PROJECT, 0)
