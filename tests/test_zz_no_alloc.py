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


def test_noalloc_in_place_and_allocates_nothing(semlib):
    """Outputs aliasing the inputs (the case where the allocating call needs
    its workspace) give the allocating call's result; after the first call
    on the device (which may load the library's device code and its static
    array), further calls leave the device's free memory unchanged; each
    call counts one FP64 apply."""
    import torch

    from schrodingersem_gb300 import capi
    L = capi.load()
    co, el = structured(10, box=(-2.0, 2.0, -2.0, 2.0), jitter=0.15, seed=9)
    ctx = semlib.Context(6, coords=co, elements=el)
    h = ctx._h
    g = torch.Generator(device="cuda").manual_seed(5)
    V = torch.rand(ctx.shape, dtype=torch.float64, device="cuda", generator=g) * 4 - 2
    qr = torch.randn(ctx.shape, dtype=torch.float64, device="cuda", generator=g)
    qi = torch.randn(ctx.shape, dtype=torch.float64, device="cuda", generator=g)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    ar, ai = qr.clone(), qi.clone()
    capi.check(L.sem_apply_schro_res(h, p(V), 0.02, p(ar), p(ai), p(ar), p(ai)), "sem_apply_schro_res")
    free = []
    for call in range(3):
        br, bi = qr.clone(), qi.clone()
        before = ctx.stats().fp64_applies
        capi.check(L.sem_apply_schro_res_noalloc(h, p(V), 0.02, p(br), p(bi), p(br), p(bi)),
                   "sem_apply_schro_res_noalloc")
        torch.cuda.synchronize()
        assert ctx.stats().fp64_applies == before + 1
        free.append(torch.cuda.mem_get_info()[0])
        for x, y in ((br, ar), (bi, ai)):
            assert _rel(x.cpu().numpy(), y.cpu().numpy()) <= TOL64
        del br, bi
        torch.cuda.synchronize()
    # the clones are freed to torch's cache, not to the device, so any drop
    # in free memory after the first call would be the entry point's own
    assert free[1] == free[2], free
