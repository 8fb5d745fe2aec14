"""Parity of the CUDA operators with the CPU oracle, through the C ABI.

Gather-scatter (unmask, global_sum, mask) is compared bit for bit; the
operator applies within 1e-12 relative in FP64 (the tolerance the hot path
is specified to), the FP32 apply within 2e-5 relative."""
import numpy as np
import pytest

from tests.util import SMALL_MESH, rel_err, structured

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


def _pair(semlib, oracle, p, kind, corrected=False):
    if kind == "small":
        ctx = semlib.Context(p, folder=SMALL_MESH, corrected_metric=corrected)
        om = oracle.Mesh(p, folder=SMALL_MESH, ref_compat=not corrected)
    else:
        co, el = structured(5 if p < 10 else 3, box=(-1.0, 2.0, -0.5, 1.5), jitter=0.2, seed=p)
        ctx = semlib.Context(p, coords=co, elements=el, corrected_metric=corrected)
        om = oracle.Mesh(p, coords=co, elements=el, ref_compat=not corrected)
    return ctx, om


CASES = [("small", p) for p in (1, 2, 3, 6, 8)] + [("jit", p) for p in range(1, 17)]


@pytest.mark.parametrize("kind,p", CASES)
def test_setup_matches(semlib, oracle, kind, p):
    ctx, om = _pair(semlib, oracle, p, kind)
    x, w, D = ctx.quadrature()
    tol = 0 if p <= 8 else 2e-15
    assert np.max(abs(x - om.x)) <= tol
    assert np.max(abs(w - om.w)) <= (0 if p <= 8 else 1e-14)
    assert np.max(abs(D - om.D)) <= (0 if p <= 8 else 1e-11 * np.max(abs(om.D)))
    J, A, B, C = ctx.metrics()
    for a, b in ((J, om.J), (A, om.A), (B, om.B), (C, om.C)):
        assert rel_err(a, b) <= (0 if p <= 8 else 1e-14)
    assert ctx.dof() == om.dof()
    X, Y = ctx.node_coords()
    OX, OY = om.node_coords()
    assert np.max(abs(X - OX)) <= 1e-15 * 4 and np.max(abs(Y - OY)) <= 1e-15 * 4


@pytest.mark.parametrize("kind,p", CASES)
def test_gather_scatter_bit_exact(semlib, oracle, kind, p):
    ctx, om = _pair(semlib, oracle, p, kind)
    rng = np.random.default_rng(100 + p)
    a = rng.standard_normal(om.shape)
    for name in ("unmask", "global_sum", "mask"):
        d = ctx.to_device(a)
        getattr(ctx, name)(d)
        got = d.cpu().numpy()
        want = getattr(om, name)(a)
        assert np.array_equal(got, want), name
    b = rng.standard_normal(om.shape)
    got = ctx.dot(ctx.to_device(a), ctx.to_device(b))
    want = om.dot(a, b)
    assert abs(got - want) <= 1e-13 * (abs(want) + np.sqrt(om.dot(a, a) * om.dot(b, b)))
    one = ctx.to_device(np.ones(om.shape))
    assert ctx.dot(one, one) == om.dof()  # mpi_tests/dot.cpp:9-33


@pytest.mark.parametrize("kind,p", CASES)
@pytest.mark.parametrize("corrected", [False, True])
def test_operators_fp64(semlib, oracle, kind, p, corrected):
    ctx, om = _pair(semlib, oracle, p, kind, corrected)
    rng = np.random.default_rng(7 * p + 3)
    u = rng.standard_normal(om.shape)
    v = rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    du, dv, dV = ctx.to_device(u), ctx.to_device(v), ctx.to_device(V)
    assert rel_err(ctx.gproj(du).cpu().numpy(), om.gproj(u)) <= TOL64
    assert rel_err(ctx.apply_laplace(du).cpu().numpy(), om.apply_laplace(u)) <= TOL64
    assert rel_err(ctx.apply_helmholtz(dV, du).cpu().numpy(), om.apply_helmholtz(V, u)) <= TOL64
    alpha = 0.0123
    yr, yi = ctx.schro_res(dV, alpha, du, dv)
    orr, oii = om.schro_res(V, alpha, u, v)
    assert rel_err(yr.cpu().numpy(), orr) <= TOL64 and rel_err(yi.cpu().numpy(), oii) <= TOL64
    yr, yi = ctx.schro_f(dV, du, dv)
    orr, oii = om.schro_f(V, u, v)
    assert rel_err(yr.cpu().numpy(), orr) <= TOL64 and rel_err(yi.cpu().numpy(), oii) <= TOL64
    # outputs are masked: applying mask again changes nothing
    out = ctx.apply_laplace(du)
    again = out.clone()
    ctx.mask(again)
    assert bool((again == out).all())


@pytest.mark.parametrize("kind,p", [("small", 3), ("small", 8), ("jit", 4), ("jit", 8), ("jit", 12), ("jit", 16)])
def test_schro_res_fp32(semlib, oracle, kind, p):
    import torch
    ctx, om = _pair(semlib, oracle, p, kind)
    rng = np.random.default_rng(p)
    u, v = rng.standard_normal(om.shape), rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    f = torch.float32
    yr, yi = ctx.schro_res_f32(ctx.to_device(V, f), 0.05, ctx.to_device(u, f), ctx.to_device(v, f))
    orr, oii = om.schro_res(V.astype(np.float32).astype(np.float64), 0.05,
                            u.astype(np.float32).astype(np.float64), v.astype(np.float32).astype(np.float64))
    assert rel_err(yr.cpu().double().numpy(), orr) <= TOL32
    assert rel_err(yi.cpu().double().numpy(), oii) <= TOL32


def test_apply_unmasked_input_uses_owner_copies(semlib, oracle):
    # galerkin_op unmasks its input: non-owner copies of shared nodes are
    # ignored, boundary copies are used as given (galerkin.hpp:24-35)
    ctx, om = _pair(semlib, oracle, 4, "small")
    rng = np.random.default_rng(5)
    u = rng.standard_normal(om.shape)
    junk = u.copy()
    shared_non_owner = (om.unmask(om.mask(np.ones(om.shape))) == 1) & (om.mask(np.ones(om.shape)) == 0)
    junk[shared_non_owner] = 1e3
    a = ctx.apply_laplace(ctx.to_device(u)).cpu().numpy()
    b = ctx.apply_laplace(ctx.to_device(junk)).cpu().numpy()
    assert rel_err(a, om.apply_laplace(u)) <= TOL64
    assert rel_err(b, om.apply_laplace(junk)) <= TOL64
    assert np.array_equal(b, ctx.apply_laplace(ctx.to_device(om.unmask(junk))).cpu().numpy())


def test_vec_axpby(semlib):
    import torch
    co, el = structured(3)
    ctx = semlib.Context(2, coords=co, elements=el)
    x = torch.randn(ctx.shape, dtype=torch.float64, device="cuda")
    y = torch.randn(ctx.shape, dtype=torch.float64, device="cuda")
    out = torch.empty_like(x)
    ctx.axpby(2.0, x, -0.5, y, out)
    torch.cuda.synchronize()
    assert torch.allclose(out, 2.0 * x + (-0.5) * y, rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("kind,p", [("small", 1), ("small", 4), ("jit", 2), ("jit", 8), ("jit", 13)])
def test_in_place_ring_assembly_matches_separate_output(semlib, oracle, kind, p):
    """outputs that do not overlap the inputs are assembled in place over the
    element rings only; outputs that alias an input go through a workspace and
    the full assembly kernel.  Both give the same bits."""
    import torch
    ctx, om = _pair(semlib, oracle, p, kind)
    rng = np.random.default_rng(40 + p)
    u, v = rng.standard_normal(om.shape), rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    dV = ctx.to_device(V)
    yr, yi = ctx.schro_res(dV, 0.03, ctx.to_device(u), ctx.to_device(v))
    ar, ai = ctx.to_device(u), ctx.to_device(v)
    ctx.schro_res(dV, 0.03, ar, ai, ar, ai)  # in place: workspace path
    assert torch.equal(yr, ar) and torch.equal(yi, ai)
    orr, oii = om.schro_res(V, 0.03, u, v)
    assert rel_err(yr.cpu().numpy(), orr) <= TOL64 and rel_err(yi.cpu().numpy(), oii) <= TOL64
    f = torch.float32
    zr, zi = ctx.schro_res_f32(ctx.to_device(V, f), 0.03, ctx.to_device(u, f), ctx.to_device(v, f))
    br, bi = ctx.to_device(u, f), ctx.to_device(v, f)
    ctx.schro_res_f32(ctx.to_device(V, f), 0.03, br, bi, br, bi)
    assert torch.equal(zr, br) and torch.equal(zi, bi)
    a = ctx.apply_laplace(ctx.to_device(u))
    b = ctx.to_device(u)
    ctx.apply_laplace(b, b)
    assert torch.equal(a, b)
    assert rel_err(a.cpu().numpy(), om.apply_laplace(u)) <= TOL64


@pytest.mark.parametrize("n,p,order", [(5, 1, "rows"), (5, 8, "rows"), (40, 4, "rows"), (24, 8, "rows"),
                                         (7, 13, "rows"), (6, 16, "rows"), (24, 8, "shuffled"),
                                         (9, 3, "shuffled")])
def test_pipelined_apply_matches_one_pass_kernel(semlib, oracle, n, p, order):
    """the bulk-copy pipelined element kernel (mesh tails loaded with plain
    loads; side pairs inside a batch summed by the kernel, the others by the
    ring pass) and the one-pass kernel give the same bits for every operator,
    in row order (most horizontal neighbours share a batch) and with the
    elements shuffled and their corners rotated (few do)"""
    import torch
    from schrodingersem_gb300 import capi
    co, el = structured(n, box=(-1.0, 2.0, -0.5, 1.5), jitter=0.2, seed=n + p)
    if order == "shuffled":
        rng = np.random.default_rng(7 * n + p)
        el = el[rng.permutation(len(el))]
        el = np.stack([np.roll(row, int(r)) for row, r in zip(el, rng.integers(0, 4, len(el)))])
    ctx = semlib.Context(p, coords=co, elements=el)
    rng = np.random.default_rng(60 + p)
    shp = ctx.shape
    u, v = ctx.to_device(rng.standard_normal(shp)), ctx.to_device(rng.standard_normal(shp))
    V = ctx.to_device(rng.uniform(-5, 5, shp))
    f = torch.float32

    def run_all():
        ctx.set_option(capi.OPT_APPLY_PIPELINE, 1)
        out = [ctx.apply_laplace(u), ctx.apply_helmholtz(V, u), ctx.gproj(u)]
        out += list(ctx.schro_res(V, 0.02, u, v)) + list(ctx.schro_f(V, u, v))
        out += list(ctx.schro_res_f32(V.to(f), 0.02, u.to(f), v.to(f)))
        torch.cuda.synchronize()
        return out

    a = run_all()
    ctx.set_option(capi.OPT_APPLY_PIPELINE, 0)
    b = [ctx.apply_laplace(u), ctx.apply_helmholtz(V, u), ctx.gproj(u)]
    b += list(ctx.schro_res(V, 0.02, u, v)) + list(ctx.schro_f(V, u, v))
    b += list(ctx.schro_res_f32(V.to(f), 0.02, u.to(f), v.to(f)))
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    if n <= 7:
        om = oracle.Mesh(p, coords=co, elements=el)
        assert rel_err(a[0].cpu().numpy(), om.apply_laplace(u.cpu().numpy())) <= TOL64


@pytest.mark.parametrize("n,p,order,corrected,neumann", [
    (5, 1, "rows", False, False), (24, 8, "rows", False, False), (24, 8, "shuffled", True, False),
    (9, 3, "shuffled", False, True), (12, 4, "rows", True, True), (7, 12, "rows", False, False),
    (6, 15, "shuffled", True, False), (40, 6, "rows", False, False)])
def test_on_the_fly_geometry_apply_fp32(semlib, oracle, n, p, order, corrected, neumann):
    """FP32 Res apply with the geometric factors computed inside the
    pipelined kernel from each element's corner differences (apply pipeline
    2): within the FP32 tolerance of the oracle's FP64 Res (include/Quad.hpp:39-54
    metrics, both metric conventions, Dirichlet and natural boundaries,
    shuffled and rotated elements, mesh tails), and close to the pipelined
    kernel that reads the stored FP32 factors"""
    import torch
    from schrodingersem_gb300 import capi
    co, el = structured(n, box=(-1.0, 2.0, -0.5, 1.5), jitter=0.2, seed=3 * n + p)
    if order == "shuffled":
        rng = np.random.default_rng(11 * n + p)
        el = el[rng.permutation(len(el))]
        el = np.stack([np.roll(row, int(r)) for row, r in zip(el, rng.integers(0, 4, len(el)))])
    ctx = semlib.Context(p, coords=co, elements=el, corrected_metric=corrected, neumann=neumann)
    om = oracle.Mesh(p, coords=co, elements=el, ref_compat=not corrected, neumann=neumann)
    rng = np.random.default_rng(70 + p)
    u, v = rng.standard_normal(om.shape), rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    f = torch.float32
    args = (ctx.to_device(V, f), 0.04, ctx.to_device(u, f), ctx.to_device(v, f))
    ctx.set_option(capi.OPT_APPLY_PIPELINE, 2)
    gr, gi = ctx.schro_res_f32(*args)
    ctx.set_option(capi.OPT_APPLY_PIPELINE, 1)
    sr, si = ctx.schro_res_f32(*args)
    torch.cuda.synchronize()
    c32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    orr, oii = om.schro_res(c32(V), 0.04, c32(u), c32(v))
    assert rel_err(gr.cpu().double().numpy(), orr) <= TOL32
    assert rel_err(gi.cpu().double().numpy(), oii) <= TOL32
    assert rel_err(gr.cpu().double().numpy(), sr.cpu().double().numpy()) <= TOL32
    assert rel_err(gi.cpu().double().numpy(), si.cpu().double().numpy()) <= TOL32
    ctx.dot(ctx.to_device(u), ctx.to_device(v))  # raises if a bounded wait of the kernel expired


def test_apply_pipeline_option_range(semlib):
    from schrodingersem_gb300 import capi
    co, el = structured(4, box=(0.0, 1.0, 0.0, 1.0), jitter=0.1, seed=1)
    ctx = semlib.Context(4, coords=co, elements=el)
    for v in (0, 1, 2):
        ctx.set_option(capi.OPT_APPLY_PIPELINE, v)
    with pytest.raises(capi.SemError):
        ctx.set_option(capi.OPT_APPLY_PIPELINE, 3)
