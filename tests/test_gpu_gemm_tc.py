"""The network's GEMM on the 5th-generation tensor cores (tcgen05.mma, FP32
accumulator in tensor memory) against a float64 product of the same BF16
operands and against the warp-level mma.sync kernel, on the network's
shapes, on ragged edges (M, N, K not multiples of the tiles) and on tiny and
K-long cases; the learner's training step gives the same gradients on both
paths, and no bounded wait expired."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(4096, 256, 324), (4096, 162, 256), (4096, 384, 324), (1000, 70, 37), (128, 64, 16), (300, 384, 1024),
          (1, 1, 1), (129, 65, 17), (2048, 256, 4096)]


def _gemm(L, path, A, B, M, N, K):
    import torch
    from schrodingersem_gb300 import capi
    capi.check(L.sem_gemm_set_path(path), "sem_gemm_set_path")
    Cm = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    capi.check(L.sem_gemm_bf16(M, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                               C.c_void_p(Cm.data_ptr()), None), "sem_gemm_bf16")
    torch.cuda.synchronize()
    return Cm


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_tcgen05_gemm_matches_fp64_and_mma_sync(semlib, M, N, K):
    import torch
    from schrodingersem_gb300 import capi
    L = capi.load()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn(K, N, generator=g, device="cuda").to(torch.bfloat16)
    ref = (A.double() @ B.double())
    scale = (A.double().abs() @ B.double().abs()).clamp_min(1e-30)
    try:
        c_tc = _gemm(L, 1, A, B, M, N, K)
        c_ms = _gemm(L, 0, A, B, M, N, K)
    finally:
        capi.check(L.sem_gemm_set_path(1), "sem_gemm_set_path")
    assert bool(torch.isfinite(c_tc).all())
    # FP32 accumulation of exact BF16 products: error well below 1e-5 of sum |a||b|
    assert float(((c_tc.double() - ref).abs() / scale).max()) < 1e-5
    assert float(((c_tc.double() - c_ms.double()).abs() / scale).max()) < 1e-5
    e = C.c_int(-1)
    capi.check(L.sem_gemm_check_error(C.byref(e)), "sem_gemm_check_error")
    assert e.value == 0


def test_learner_gradients_same_on_both_paths(semlib):
    """one training step's loss and gradients with the tcgen05 GEMMs equal
    the mma.sync ones to FP32 summation-order differences"""
    import torch
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    L = capi.load()
    rng = np.random.default_rng(3)
    X = torch.tensor(rng.standard_normal((700, 100)), dtype=torch.bfloat16, device="cuda")
    T = torch.tensor(rng.standard_normal((700, 50)), dtype=torch.float32, device="cuda")
    out = {}
    try:
        for path in (0, 1):
            capi.check(L.sem_gemm_set_path(path), "sem_gemm_set_path")
            net = Learner(100, 96, 50, seed=5)
            loss = net.train_step(X, T, lr=0.0)
            out[path] = (loss, [net.grads(l) for l in range(3)])
    finally:
        capi.check(L.sem_gemm_set_path(1), "sem_gemm_set_path")
    assert abs(out[0][0] - out[1][0]) <= 1e-5 * abs(out[0][0])
    for l in range(3):
        for a, b in zip(out[0][1][l], out[1][1][l]):
            assert np.abs(a - b).max() <= 1e-4 * max(np.abs(a).max(), 1e-12)


@pytest.mark.parametrize("rows,d_in,hidden,d_out", [(4096, 324, 256, 162), (1000, 100, 96, 50), (129, 676, 256, 256),
                                                    (1, 36, 16, 18), (300, 324, 200, 162)])
def test_fused_forward_matches_per_layer_gemms(semlib, rows, d_in, hidden, d_out):
    """the one-launch inference pass (three layers chained through tensor
    memory and shared memory) against the per-layer tcgen05 GEMMs with their
    BF16 activations in global memory, and against the mma.sync kernel"""
    import torch
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.learned import Learner
    L = capi.load()
    g = torch.Generator(device="cuda").manual_seed(rows + d_in + hidden + d_out)
    X = torch.randn(rows, d_in, generator=g, device="cuda").to(torch.bfloat16)
    net = Learner(d_in, hidden, d_out, seed=9)
    out = {}
    try:
        for path in (1, 2, 0):
            capi.check(L.sem_gemm_set_path(path), "sem_gemm_set_path")
            out[path] = net.forward(X).double()
            torch.cuda.synchronize()
    finally:
        capi.check(L.sem_gemm_set_path(1), "sem_gemm_set_path")
    scale = out[2].abs().max().clamp_min(1e-30)
    assert bool(torch.isfinite(out[1]).all())
    assert float((out[1] - out[2]).abs().max() / scale) < 1e-5
    # mma.sync rounds the same products in another order; a BF16 hidden value
    # may then round to its neighbour
    assert float((out[1] - out[0]).abs().max() / scale) < 2e-2
    e = C.c_int(-1)
    capi.check(L.sem_gemm_check_error(C.byref(e)), "sem_gemm_check_error")
    assert e.value == 0
