"""sem_apply_schro_res_noalloc: the Res operator for callers that cannot let
the library allocate device memory (its intermediate lives in a static
device array).  It must give the same result as sem_apply_schro_res, call
after call, whether it runs first in a fresh process or after the other
tests.  Kept in its own file, collected last."""
import ctypes as C

import numpy as np
import pytest

from tests.util import structured

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _rel(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)


def test_noalloc_matches_allocating_apply_twice(semlib):
    import torch

    from schrodingersem_gb300 import capi
    L = capi.load()
    co, el = structured(12, box=(-3.0, 3.0, -3.0, 3.0), jitter=0.1, seed=4)
    ctx = semlib.Context(7, coords=co, elements=el)
    h = ctx._h
    shape = ctx.shape
    assert 2 * ctx.n <= (1 << 20)
    g = torch.Generator(device="cuda").manual_seed(11)
    for call in range(2):
        V = torch.rand(shape, dtype=torch.float64, device="cuda", generator=g) * 10 - 5
        qr = torch.randn(shape, dtype=torch.float64, device="cuda", generator=g)
        qi = torch.randn(shape, dtype=torch.float64, device="cuda", generator=g)
        alpha = 0.01 * (call + 1)
        ar, ai = torch.empty_like(qr), torch.empty_like(qr)
        br, bi = torch.full_like(qr, np.nan), torch.full_like(qr, np.nan)
        p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        capi.check(L.sem_apply_schro_res(h, p(V), alpha, p(qr), p(qi), p(ar), p(ai)), "sem_apply_schro_res")
        capi.check(L.sem_apply_schro_res_noalloc(h, p(V), alpha, p(qr), p(qi), p(br), p(bi)),
                   "sem_apply_schro_res_noalloc")
        torch.cuda.synchronize()
        for x, y in ((br, ar), (bi, ai)):
            x, y = x.cpu().numpy(), y.cpu().numpy()
            assert np.all(np.isfinite(x))
            assert _rel(x, y) <= TOL64


def test_noalloc_rejects_meshes_above_capacity(semlib):
    import torch

    from schrodingersem_gb300 import capi
    L = capi.load()
    co, el = structured(48, jitter=0.0)
    ctx = semlib.Context(16, coords=co, elements=el)  # 2 * 2304 * 289 > 2^20
    assert 2 * ctx.n > (1 << 20)
    t = torch.zeros(ctx.shape, dtype=torch.float64, device="cuda")
    p = C.c_void_p(t.data_ptr())
    st = L.sem_apply_schro_res_noalloc(ctx._h, p, 0.1, p, p, p, p)
    assert st == 6  # SEM_ERR_UNSUPPORTED
    assert b"static capacity" in L.sem_last_error()
