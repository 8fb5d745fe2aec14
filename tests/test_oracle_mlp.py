"""CPU pins of the network oracle (oracle/mlp.py): BF16 rounding and
backpropagation against finite differences."""
import numpy as np

from oracle import mlp


def _params(rng, d_in, H, d_out):
    return [(rng.standard_normal((i, o)).astype(np.float32) / np.sqrt(i), rng.standard_normal(o).astype(np.float32) * 0.1)
            for i, o in ((d_in, H), (H, H), (H, d_out))]


def test_bf16_round_known_values():
    vals = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -7 + 2.0 ** -9, -2.5, 0.0,
                     3.0e38, 1.0e-40], np.float32)
    got = mlp.bf16_round(vals)
    # 1+2^-8 is a tie -> even (1.0); 1+3*2^-8 is a tie -> even (1+2^-6)
    want = np.array([1.0, 1.0, 1.0 + 2.0 ** -6, 1.0 + 2.0 ** -7, -2.5, 0.0], np.float32)
    assert np.array_equal(got[:6], want)
    # finite large value stays within one BF16 step; denormals keep their sign and scale
    assert abs(got[6] - vals[6]) <= 2.0 ** -8 * vals[6]
    assert got[7] >= 0


def test_fp64_backprop_matches_finite_differences():
    rng = np.random.default_rng(3)
    d_in, H, d_out, rows = 6, 8, 5, 7
    x = rng.standard_normal((rows, d_in))
    t = rng.standard_normal((rows, d_out))
    params = [(W.astype(np.float64), b.astype(np.float64)) for W, b in _params(rng, d_in, H, d_out)]
    g = mlp.grads_fp64(x, t, params)
    h = 1e-6
    for l in range(3):
        W, b = params[l]
        for (arr, ga) in ((W, g[l][0]), (b, g[l][1])):
            for idx in [tuple(rng.integers(0, s) for s in arr.shape) for _ in range(6)]:
                old = arr[idx]
                arr[idx] = old + h
                lp = mlp.loss_fp64(x, t, params)
                arr[idx] = old - h
                lm = mlp.loss_fp64(x, t, params)
                arr[idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - ga[idx]) <= 1e-6 * max(1.0, abs(fd)), (l, idx, fd, ga[idx])


def test_bf16_backprop_close_to_fp64():
    rng = np.random.default_rng(4)
    d_in, H, d_out, rows = 32, 48, 16, 64
    x = mlp.bf16_round(rng.standard_normal((rows, d_in)).astype(np.float32))
    t = rng.standard_normal((rows, d_out)).astype(np.float32)
    params = _params(rng, d_in, H, d_out)
    loss, g = mlp.loss_and_grads(x, t, params, bf16=False)
    g64 = mlp.grads_fp64(x, t, params)
    assert abs(loss - mlp.loss_fp64(x, t, params)) < 1e-5 * loss
    for l in range(3):
        for a, b in zip(g[l], g64[l]):
            assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    # BF16 operands (8-bit significands) move the gradients by a few percent
    # of their norm; a sanity bound only (the GPU is checked against the BF16
    # restatement itself)
    loss_b, gb = mlp.loss_and_grads(x, t, params, bf16=True)
    for l in range(3):
        for a, b in zip(gb[l], g64[l]):
            assert np.linalg.norm(a - b) <= 0.15 * np.linalg.norm(b)


def test_adam_first_step_moves_by_lr():
    w = np.ones(4, np.float32)
    g = np.array([1.0, -2.0, 0.5, 0.0], np.float32)
    w2, m, v = mlp.adam_update(w, g, np.zeros(4, np.float32), np.zeros(4, np.float32), 1, 1e-2)
    # first step: m/c1 = g, sqrt(v/c2) = |g|  ->  w - lr sign(g)
    assert np.allclose(w2[:3], w[:3] - 1e-2 * np.sign(g[:3]), atol=1e-6)
    assert w2[3] == w[3]
