"""Failure detection without a GPU fault.

Every failure here is made on the host or by a bounded device-side wait
running out; none faults, traps or hangs the GPU:
  * a grid-barrier wait of the persistent solver given a 1 ns limit expires,
    the call returns SEM_ERR_DEVICE_WAIT and the same context then solves
    normally, to the bits of a fresh context;
  * a NaN in the initial state (injected on the host) makes the stage solve
    fail to converge within max_iter: the driver reports failure, as the
    reference does (include/minres.hpp:92-106, include/openmp_impl/
    schrodinger.hpp:223-226), and returns;
  * truncated or missing mesh files give SEM_ERR_IO (include/load_mesh.hpp:
    92-118 throws in the same places), corner ids out of range and elements
    that repeat a corner give SEM_ERR_MESH;
  * a non-positive time step is rejected before any step (the reference's
    `while (t < T)` with `t += dt` would never end);
  * a network whose predictions are NaN leaves the learned stage guess on
    its fallback, the extrapolation, and the run matches the extrapolated
    run bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

from tests.util import SMALL_MESH, structured

pytestmark = pytest.mark.gpu

SEM_ERR_ARG, SEM_ERR_MESH, SEM_ERR_IO, SEM_ERR_DEVICE_WAIT = 1, 3, 4, 5


def _packet_case(semlib, n=16, p=6):
    from schrodingersem_gb300.meshgen import gaussian_packet
    co, el = structured(n, box=(-4.0, 4.0, -4.0, 4.0), jitter=0.1, seed=3)
    ctx = semlib.Context(p, coords=co, elements=el)
    X, Y = ctx.node_coords()
    re, im = gaussian_packet(X, Y, (-1.0, 0.0), 1.0, (2.0, 0.0))
    return ctx, re, im, 0.5 * (X * X + Y * Y), (co, el)


def _solve(ctx, V, b_re, b_im, tol=1e-10):
    from schrodingersem_gb300 import capi
    L = capi.load()
    xr, xi = ctx.zeros(), ctx.zeros()
    r = capi.SemSolverResults()
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = L.sem_minres_schro(ctx._h, p(V), 0.01, p(xr), p(xi), p(b_re), p(b_im), 20 * ctx.dof(), tol, 1,
                            C.byref(r))
    return st, r, xr, xi


def test_grid_barrier_limit_expires_and_context_recovers(semlib):
    import torch

    from schrodingersem_gb300 import capi
    ctx, re, im, V, (co, el) = _packet_case(semlib)
    dV = ctx.to_device(V)
    b_re, b_im = ctx.gproj(ctx.to_device(re)), ctx.gproj(ctx.to_device(im))
    ctx.set_option(capi.OPT_WAIT_TIMEOUT_MS, 1e-6)  # 1 ns: every real wait runs out
    st, _, _, _ = _solve(ctx, dV, b_re, b_im)
    torch.cuda.synchronize()
    assert st == SEM_ERR_DEVICE_WAIT, st
    assert b"timed out" in capi.load().sem_last_error()
    ctx.set_option(capi.OPT_WAIT_TIMEOUT_MS, 2000.0)
    st, r, xr, xi = _solve(ctx, dV, b_re, b_im)
    assert st == 0 and r.success
    fresh = semlib.Context(6, coords=co, elements=el)
    st2, r2, yr, yi = _solve(fresh, fresh.to_device(V), fresh.gproj(fresh.to_device(re)),
                             fresh.gproj(fresh.to_device(im)))
    assert st2 == 0 and r2.success and r2.n_iter == r.n_iter
    assert torch.equal(xr, yr) and torch.equal(xi, yi)


@pytest.mark.parametrize("method", ["bdf2", "dirk4s3", "dirk4s5"])
def test_nan_state_fails_without_hanging(semlib, method):
    ctx, re, im, V, _ = _packet_case(semlib, n=6, p=4)
    re = re.copy()
    re[3, 2, 2] = np.nan
    ok = ctx.schrodinger(method, re, im.copy(), V, 0.05, 0.01, 200, 1e-10)
    assert not ok
    st = ctx.stats()
    assert st.last_stage_iters[0] == 201  # max_iter + 1: not converged (minres.hpp:102-106)


def test_nan_rhs_minres_reports_nonconvergence(semlib):
    ctx, re, im, V, _ = _packet_case(semlib, n=6, p=4)
    b = ctx.to_device(re)
    b[0, 1, 1] = float("nan")
    xr, xi = ctx.zeros(), ctx.zeros()
    ok, it, res = ctx.minres_schro(ctx.to_device(V), 0.01, xr, xi, b, ctx.to_device(im), 50, 1e-10, x_is_zero=True)
    assert not ok and it == 51 and not np.isfinite(res)


def test_bad_mesh_files_return_io_errors(semlib, tmp_path):
    from schrodingersem_gb300 import capi
    L = capi.load()
    src = {f: open(os.path.join(SMALL_MESH, f)).read() for f in ("info.txt", "coordinates.txt", "elements.txt")}

    def load(files):
        d = tmp_path / f"m{len(list(tmp_path.iterdir()))}"
        d.mkdir()
        for name, text in files.items():
            (d / name).write_text(text)
        h = C.c_void_p()
        st = L.sem_ctx_load(C.byref(h), 3, str(d).encode(), 0)
        if st == 0:
            L.sem_ctx_destroy(h)
        return st

    assert load(src) == 0
    truncated = dict(src, **{"elements.txt": "\n".join(src["elements.txt"].splitlines()[:20])})
    assert load(truncated) == SEM_ERR_IO
    assert b"elements.txt" in L.sem_last_error()
    assert load({k: v for k, v in src.items() if k != "coordinates.txt"}) == SEM_ERR_IO
    assert load(dict(src, **{"coordinates.txt": "0.0 1.0\n2.0"})) == SEM_ERR_IO
    assert load(dict(src, **{"info.txt": "garbage"})) == SEM_ERR_IO
    assert L.sem_ctx_load(C.byref(C.c_void_p()), 3, str(tmp_path / "absent").encode(), 0) == SEM_ERR_IO
    lines = src["elements.txt"].splitlines()
    assert load(dict(src, **{"elements.txt": "\n".join(["0 1 2 9999"] + lines[1:])})) == SEM_ERR_MESH
    assert load(dict(src, **{"elements.txt": "\n".join(["0 1 1 2"] + lines[1:])})) == SEM_ERR_MESH


@pytest.mark.parametrize("method", ["bdf2", "dirk4s3", "dirk4s5"])
def test_non_positive_dt_is_rejected(semlib, method):
    from schrodingersem_gb300.capi import SemError
    ctx, re, im, V, _ = _packet_case(semlib, n=2, p=2)
    for dt in (0.0, -1e-3, float("nan")):
        with pytest.raises(SemError) as e:
            ctx.schrodinger(method, re.copy(), im.copy(), V, 1.0, dt, 100, 1e-10)
        assert e.value.status == SEM_ERR_ARG


def test_nan_network_falls_back_to_extrapolation(semlib):
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    ctx, re, im, V, _ = _packet_case(semlib, n=6, p=5)
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    L = Learner.for_mesh(ctx.N, hidden=32, seed=1)
    W, b = L.params(2)
    L.set_params(2, np.full_like(W, np.nan), b)
    ctx.set_learner(L)
    dt, steps = 0.01, 5
    runs = {}
    for guess in (capi.GUESS_EXTRAPOLATE, capi.GUESS_LEARNED):
        ctx.set_option(capi.OPT_STAGE_GUESS, guess)
        a, c = re.copy(), im.copy()
        s0 = ctx.stats()
        for _ in range(steps):
            assert ctx.schrodinger("dirk4s3", a, c, V, 0.5 * dt, dt, 20 * ctx.dof(), 1e-10)
        s1 = ctx.stats()
        runs[guess] = (a, c, s1.learned_guesses - s0.learned_guesses, s1.learned_accepted - s0.learned_accepted)
    a, c, n_guess, n_acc = runs[capi.GUESS_LEARNED]
    assert n_guess == 3 * (steps - 2) and n_acc == 0
    assert np.array_equal(a, runs[capi.GUESS_EXTRAPOLATE][0]) and np.array_equal(c, runs[capi.GUESS_EXTRAPOLATE][1])
