"""Learned stage guess: the BF16 tensor-core network against the CPU
restatement (oracle/mlp.py), and the SDIRK driver with the network in the
loop (states agree with FP64 to 1e-8; the network's guesses are checked
against the extrapolation's FP64 residual)."""
import numpy as np
import pytest

from tests.util import rel_err, structured

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_mod(semlib):
    import torch
    return torch


def _bf16(torch, a):
    return torch.as_tensor(np.asarray(a, np.float32), device="cuda").to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (7, 13, 3), (130, 67, 33), (64, 64, 32), (257, 200, 520)])
def test_gemm_bf16_matches_oracle(semlib, torch_mod, M, N, K):
    from oracle import mlp
    from schrodingersem_gb300.learned import gemm_bf16
    torch = torch_mod
    rng = np.random.default_rng(M * 1000 + N + K)
    A = mlp.bf16_round(rng.standard_normal((M, K)).astype(np.float32))
    B = mlp.bf16_round(rng.standard_normal((K, N)).astype(np.float32))
    Cg = gemm_bf16(_bf16(torch, A), _bf16(torch, B)).cpu().numpy()
    ref = A.astype(np.float64) @ B.astype(np.float64)
    # operands are exact BF16 values: only the FP32 accumulation differs
    scale = np.sqrt(K) * np.abs(A).max() * np.abs(B).max()
    assert np.abs(Cg - ref).max() <= 4e-7 * scale * max(1.0, np.sqrt(K) / 4)


def _net(semlib, rng, d_in, H, d_out):
    from schrodingersem_gb300.learned import Learner
    L = Learner(d_in, H, d_out, seed=5)
    params = [L.params(l) for l in range(3)]
    # non-zero biases exercise the bias paths
    for l in range(3):
        W, b = params[l]
        b = (0.1 * rng.standard_normal(b.shape)).astype(np.float32)
        L.set_params(l, W, b)
        params[l] = (W, b)
    return L, params


def test_learner_forward_and_gradients_match_oracle(semlib, torch_mod):
    from oracle import mlp
    torch = torch_mod
    rng = np.random.default_rng(9)
    d_in, H, d_out, rows = 36, 96, 20, 100
    L, params = _net(semlib, rng, d_in, H, d_out)
    x = mlp.bf16_round(rng.standard_normal((rows, d_in)).astype(np.float32))
    t = rng.standard_normal((rows, d_out)).astype(np.float32)
    xd, td = _bf16(torch, x), torch.as_tensor(t, device="cuda")
    out = L.forward(xd).cpu().numpy()
    ref_out, _ = mlp.forward(x, params, bf16=True)
    assert rel_err(out, ref_out) < 1e-3
    loss = L.train_step(xd, td, lr=0.0)
    ref_loss, ref_g = mlp.loss_and_grads(x, t, params, bf16=True)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    for l in range(3):
        gW, gb = L.grads(l)
        # BF16 operands are the same on both sides; the FP32 accumulation order
        # and rare one-step BF16 rounding flips of intermediates remain
        assert rel_err(gW, ref_g[l][0]) < 5e-3, l
        assert rel_err(gb, ref_g[l][1]) < 5e-3, l
    # the parameters did not move (lr = 0)
    for l in range(3):
        W, b = L.params(l)
        assert np.array_equal(W, params[l][0]) and np.array_equal(b, params[l][1])


def test_adam_step_matches_oracle(semlib, torch_mod):
    from oracle import mlp
    torch = torch_mod
    rng = np.random.default_rng(10)
    d_in, H, d_out, rows = 24, 64, 12, 70
    L, params = _net(semlib, rng, d_in, H, d_out)
    x = mlp.bf16_round(rng.standard_normal((rows, d_in)).astype(np.float32))
    t = rng.standard_normal((rows, d_out)).astype(np.float32)
    lr = 1e-3
    L.train_step(_bf16(torch, x), torch.as_tensor(t, device="cuda"), lr=lr)
    for l in range(3):
        gW, gb = L.grads(l)
        W1, b1 = L.params(l)
        for new, old, g in ((W1, params[l][0], gW), (b1, params[l][1], gb)):
            want, _, _ = mlp.adam_update(old, g, np.zeros_like(g), np.zeros_like(g), 1, lr)
            assert np.allclose(new - old, want - old, rtol=1e-3, atol=1e-9), l


def test_fit_learns_a_linear_map(semlib, torch_mod):
    torch = torch_mod
    from schrodingersem_gb300.learned import Learner
    rng = np.random.default_rng(12)
    d_in, d_out, rows = 16, 8, 4096
    R = rng.standard_normal((d_in, d_out)).astype(np.float32) / 4
    x = rng.standard_normal((rows, d_in)).astype(np.float32)
    X = _bf16(torch, x)
    T = torch.as_tensor(X.float().cpu().numpy() @ R, device="cuda")
    L = Learner(d_in, 64, d_out, seed=2)
    l0 = L.train_step(X[:512].contiguous(), T[:512].contiguous(), lr=0.0)
    loss = L.fit(X, T, epochs=30, batch=256, lr=2e-3, seed=4)
    assert loss < 0.05 * l0


def _case(semlib, n=8, p=6):
    from schrodingersem_gb300.meshgen import gaussian_packet
    co, el = structured(n, box=(-4, 4, -4, 4), jitter=0.1, seed=2)
    ctx = semlib.Context(p, coords=co, elements=el)
    X, Y = ctx.node_coords()

    def packet(c, s, k):
        return gaussian_packet(X, Y, c, s, k)
    return ctx, packet, X * X + Y * Y


def test_learned_stage_guess_in_driver(semlib, torch_mod):
    """record rows from training trajectories, fit, then step a held-out
    packet: the states match the FP64 zero-guess run to 1e-8, the network is
    consulted at every stage from the third step on, and the accepted guesses
    leave a smaller residual than the extrapolation"""
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    torch = torch_mod
    ctx, packet, V = _case(semlib)
    dt, tol, steps = 0.01, 1e-10, 6
    maxit = 20 * ctx.dof()
    test_pk = ((-1.0, 0.5), 0.8, (3.0, -1.0))
    a_re, a_im = packet(*test_pk)
    assert ctx.schrodinger("dirk4s3", a_re, a_im, V, (steps - 0.5) * dt, dt, maxit, tol)
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
    train = [((-2.0, 1.0), 1.0, (2.0, 1.0)), ((1.0, -1.0), 0.7, (-3.0, 2.0)), ((0.5, 1.5), 1.2, (1.0, -3.0))]
    n_train = 8
    ctx.record(ctx.E * 3 * (n_train - 2) * len(train))
    for pk in train:
        re, im = packet(*pk)
        assert ctx.schrodinger("dirk4s3", re, im, V, (n_train - 0.5) * dt, dt, maxit, tol)
    X, T = ctx.dataset()
    assert X.shape == (ctx.E * 3 * (n_train - 2) * len(train), 4 * ctx.N ** 2)
    assert T.shape == (X.shape[0], 2 * ctx.N ** 2)
    assert torch.isfinite(T).all() and torch.isfinite(X.float()).all()
    ctx.record(0)
    L = Learner.for_mesh(ctx.N, hidden=128, seed=3)
    L.fit(X, T, epochs=20, batch=256, lr=1e-3, seed=5)
    ctx.set_learner(L)
    its = {}
    for guess in (capi.GUESS_EXTRAPOLATE, capi.GUESS_LEARNED):
        ctx.set_option(capi.OPT_STAGE_GUESS, guess)
        s0 = ctx.stats()
        b_re, b_im = packet(*test_pk)
        tot = []
        for _ in range(steps):
            assert ctx.schrodinger("dirk4s3", b_re, b_im, V, 0.5 * dt, dt, maxit, tol)
            st = ctx.stats()
            tot.append(sum(st.last_stage_iters[k] for k in range(st.last_step_stages)))
        its[guess] = tot
        assert max(rel_err(b_re, a_re), rel_err(b_im, a_im)) < 1e-8
    s1 = ctx.stats()
    assert s1.learned_guesses - s0.learned_guesses == 3 * (steps - 2)
    assert s1.learned_accepted > s0.learned_accepted
    assert 0.0 <= s1.last_guess_residual_ratio <= 1.0
    ext, lrn = its[capi.GUESS_EXTRAPOLATE], its[capi.GUESS_LEARNED]
    n_l = s1.learned_guesses - s0.learned_guesses
    mean_ratio = (s1.learned_ratio_sum - s0.learned_ratio_sum) / n_l
    print("extrapolated", ext, "learned", lrn, "accepted", s1.learned_accepted - s0.learned_accepted,
          "mean residual ratio", mean_ratio, "last theta", s1.last_guess_theta)
    # what the network gains over the extrapolation alone on this fixed-step
    # case: a stage guess with a clearly smaller FP64 residual at every stage
    # where it runs (steps 3..; measured 0.69 of the extrapolation's).  The
    # iteration count does not follow here (measured 504 against 494 over
    # steps 3..6), so the test only bounds the extra iterations at 5 %
    assert mean_ratio < 0.9
    assert sum(lrn[2:]) <= 1.05 * sum(ext[2:])


def test_learned_guess_in_adaptive_driver(semlib, torch_mod, oracle):
    """adaptive SDIRK4-5 with the network: rows are recorded from the
    adaptive run's stages, the fitted network corrects every stage guess
    after the first accepted step, and the state still equals the oracle's
    fixed-step replay of the accepted dt sequence to 1e-8"""
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    ctx, packet, V = _case(semlib)
    T, tol, err_tol, dt0 = 0.08, 1e-12, 1e-6, 0.02
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_EXTRAPOLATE)
    ctx.record(ctx.E * 5 * 40)
    for pk in (((-2.0, 1.0), 1.0, (2.0, 1.0)), ((1.0, -1.0), 0.7, (-3.0, 2.0))):
        re, im = packet(*pk)
        ok, dts, _ = ctx.schrodinger_adaptive(re, im, V, T, dt0, 100000, tol, err_tol)
        assert ok and len(dts) >= 2
    X, Tt = ctx.dataset()
    ctx.record(0)
    assert X.shape[0] > 0 and X.shape[0] % ctx.E == 0
    assert X.shape[1] == 4 * ctx.N ** 2 and Tt.shape == (X.shape[0], 2 * ctx.N ** 2)
    assert torch_mod.isfinite(Tt).all()
    L = Learner.for_mesh(ctx.N, hidden=64, seed=3)
    L.fit(X, Tt, epochs=10, batch=256, lr=1e-3, seed=5)
    ctx.set_learner(L)
    re0, im0 = packet((-1.0, 0.5), 0.8, (3.0, -1.0))
    # the same held-out packet with the scaled previous stage alone
    e0 = ctx.stats()
    ok, dts_e, nrej_e = ctx.schrodinger_adaptive(re0.copy(), im0.copy(), V, T, dt0, 100000, tol, err_tol)
    e1 = ctx.stats()
    assert ok
    ctx.set_option(capi.OPT_STAGE_GUESS, capi.GUESS_LEARNED)
    a, b = re0.copy(), im0.copy()
    s0 = ctx.stats()
    ok, dts, nrej = ctx.schrodinger_adaptive(a, b, V, T, dt0, 100000, tol, err_tol)
    s1 = ctx.stats()
    it_e = (e1.solver_iterations_fp32 - e0.solver_iterations_fp32) / (5 * (len(dts_e) + nrej_e))
    it_l = (s1.solver_iterations_fp32 - s0.solver_iterations_fp32) / (5 * (len(dts) + nrej))
    mean_ratio = (s1.learned_ratio_sum - s0.learned_ratio_sum) / max(1, s1.learned_guesses - s0.learned_guesses)
    print("inner iterations per stage: scaled previous stage", it_e, "learned", it_l, "steps", len(dts_e),
          len(dts), "mean residual ratio", mean_ratio)
    # what the network gains here: a guess residual clearly below the scaled
    # previous stage's (measured 0.65 of it) and fewer inner iterations per
    # stage (measured 22.1 against 22.8; every kernel on this path reduces
    # in a fixed order and the training is seeded, so the counts repeat)
    assert mean_ratio < 0.8
    assert it_l < it_e
    assert ok and len(dts) >= 2
    assert abs(dts.sum() - T) < 1e-12
    n_l = s1.learned_guesses - s0.learned_guesses
    assert 5 * (len(dts) - 1) <= n_l <= 5 * (len(dts) - 1 + nrej)
    assert 0.0 <= s1.last_guess_residual_ratio <= 1.0
    co, el = structured(8, box=(-4, 4, -4, 4), jitter=0.1, seed=2)  # the mesh of _case
    om = oracle.Mesh(ctx.p, coords=co, elements=el)
    r, i = re0.copy(), im0.copy()
    for d in dts:
        r, i, okk = om.schrodinger("dirk4s5", r, i, V, 0.5 * d, d, 100000, 1e-13)
        assert okk
    assert max(rel_err(a, r), rel_err(b, i)) < 1e-8


def test_set_learner_checks_shape(semlib):
    from schrodingersem_gb300.capi import SemError
    from schrodingersem_gb300.learned import Learner
    ctx, _, _ = _case(semlib, n=2, p=3)
    with pytest.raises(SemError):
        ctx.set_learner(Learner(10, 16, 5))
    ctx.set_learner(Learner.for_mesh(ctx.N, hidden=16))
    ctx.set_learner(None)
