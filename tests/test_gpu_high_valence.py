"""A corner node shared by more elements than the per-corner copy tables
hold (CORNER_NB_MAX = 8): a star of ten quads around one vertex.  The
gathers of that node fall back to the corner CSR; assembly stays bit-exact
against the CPU oracle, the operators within their tolerances, the pipelined
FP32 apply bit-identical to the one-pass kernel, and the preconditioned
mixed-precision driver within the solver's accuracy of the FP64 driver."""
import numpy as np
import pytest

from tests.util import rel_err

pytestmark = pytest.mark.gpu


def star_mesh(k=10):
    """vertex 0 at the origin, k vertices on the unit circle and k further
    out between them; element i = (centre, p_i, q_i, p_{i+1}), counter-
    clockwise, so the centre is shared by all k elements"""
    pts = [(0.0, 0.0)]
    pts += [(np.cos(2 * np.pi * i / k), np.sin(2 * np.pi * i / k)) for i in range(k)]
    pts += [(1.6 * np.cos(2 * np.pi * (i + 0.5) / k), 1.6 * np.sin(2 * np.pi * (i + 0.5) / k)) for i in range(k)]
    el = [(0, 1 + i, 1 + k + i, 1 + (i + 1) % k) for i in range(k)]
    return np.array(pts, dtype=np.float64), np.array(el, dtype=np.int32)


def _pair(semlib, oracle, p):
    co, el = star_mesh()
    return semlib.Context(p, coords=co, elements=el), oracle.Mesh(p, coords=co, elements=el)


@pytest.mark.parametrize("p", [2, 5, 8])
def test_star_gather_scatter_bit_exact(semlib, oracle, p):
    ctx, om = _pair(semlib, oracle, p)
    rng = np.random.default_rng(300 + p)
    a = rng.standard_normal(om.shape)
    for name in ("unmask", "global_sum", "mask"):
        d = ctx.to_device(a)
        getattr(ctx, name)(d)
        assert np.array_equal(d.cpu().numpy(), getattr(om, name)(a)), name
    one = ctx.to_device(np.ones(om.shape))
    assert ctx.dot(one, one) == om.dof()


@pytest.mark.parametrize("p", [2, 5, 8])
def test_star_operators(semlib, oracle, p):
    import torch
    from schrodingersem_gb300 import capi
    ctx, om = _pair(semlib, oracle, p)
    rng = np.random.default_rng(310 + p)
    u, v = rng.standard_normal(om.shape), rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    yr, yi = ctx.schro_res(ctx.to_device(V), 0.03, ctx.to_device(u), ctx.to_device(v))
    orr, oii = om.schro_res(V, 0.03, u, v)
    assert rel_err(yr.cpu().numpy(), orr) <= 1e-12 and rel_err(yi.cpu().numpy(), oii) <= 1e-12
    f = torch.float32
    args = (ctx.to_device(V, f), 0.03, ctx.to_device(u, f), ctx.to_device(v, f))
    zr, zi = ctx.schro_res_f32(*args)
    ctx.set_option(capi.OPT_APPLY_PIPELINE, 0)
    wr, wi = ctx.schro_res_f32(*args)
    assert torch.equal(zr, wr) and torch.equal(zi, wi)
    assert rel_err(zr.cpu().double().numpy(), orr) <= 2e-5 and rel_err(zi.cpu().double().numpy(), oii) <= 2e-5


def test_star_mixed_driver_matches_fp64(semlib, oracle):
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.meshgen import gaussian_packet
    ctx, _ = _pair(semlib, oracle, 6)
    X, Y = ctx.node_coords()
    re, im = gaussian_packet(X, Y, (0.2, -0.1), 0.4, (2.0, 1.0))
    V = 3.0 * (X * X + Y * Y)
    T, steps, tol = 0.02, 4, 1e-10
    a_re, a_im = re.copy(), im.copy()
    assert ctx.schrodinger("dirk4s3", a_re, a_im, V, T, T / steps, 20 * ctx.dof(), tol)
    ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
    ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
    b_re, b_im = re.copy(), im.copy()
    assert ctx.schrodinger("dirk4s3", b_re, b_im, V, T, T / steps, 20 * ctx.dof(), tol)
    assert max(rel_err(b_re, a_re), rel_err(b_im, a_im)) < 1e-8
