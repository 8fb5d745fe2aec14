"""Boundary data on the GPU (no counterpart in the reference, whose masks
zero every boundary copy: include/mask_side.hpp:28-30), through the C ABI.

  * SEM_FLAG_NEUMANN contexts against the oracle's natural-boundary mesh:
    gather-scatter bit for bit, FP64 operators within 1e-12, the FP32
    pipelined apply within 2e-5, and Schroedinger steps (FP64 and the
    element-preconditioned mixed form) within the solver tolerance;
  * sem_poisson_bc / sem_helmholtz_bc with Dirichlet data against the
    reference's own lifting (tests/golden/ref/bc_dirichlet.npz) and with
    Neumann data against the oracle; manufactured solutions for both."""
import numpy as np
import pytest

from tests.test_oracle_boundary import dudn_sides, harmonic
from tests.util import SMALL_MESH, load_ref_fixture, rel_err, structured

pytestmark = pytest.mark.gpu


def _pair(semlib, oracle, p, kind):
    if kind == "small":
        return (semlib.Context(p, folder=SMALL_MESH, neumann=True),
                oracle.Mesh(p, folder=SMALL_MESH, neumann=True))
    co, el = structured(5, box=(-1.0, 2.0, -0.5, 1.5), jitter=0.2, seed=p)
    return (semlib.Context(p, coords=co, elements=el, neumann=True),
            oracle.Mesh(p, coords=co, elements=el, neumann=True))


@pytest.mark.parametrize("kind,p", [("small", 1), ("small", 3), ("small", 8), ("jit", 2), ("jit", 6), ("jit", 12)])
def test_neumann_gather_scatter_and_operators(semlib, oracle, kind, p):
    ctx, om = _pair(semlib, oracle, p, kind)
    assert ctx.dof() == om.dof()
    rng = np.random.default_rng(30 + p)
    a = rng.standard_normal(om.shape)
    for name in ("unmask", "global_sum", "mask"):
        d = ctx.to_device(a)
        getattr(ctx, name)(d)
        assert np.array_equal(d.cpu().numpy(), getattr(om, name)(a)), name
    one = ctx.to_device(np.ones(om.shape))
    assert ctx.dot(one, one) == om.dof()
    u, v = rng.standard_normal(om.shape), rng.standard_normal(om.shape)
    V = rng.uniform(-5, 5, om.shape)
    du, dv, dV = ctx.to_device(u), ctx.to_device(v), ctx.to_device(V)
    assert rel_err(ctx.gproj(du).cpu().numpy(), om.gproj(u)) <= 1e-12
    assert rel_err(ctx.apply_laplace(du).cpu().numpy(), om.apply_laplace(u)) <= 1e-12
    assert rel_err(ctx.apply_helmholtz(dV, du).cpu().numpy(), om.apply_helmholtz(V, u)) <= 1e-12
    yr, yi = ctx.schro_res(dV, 0.0123, du, dv)
    orr, oii = om.schro_res(V, 0.0123, u, v)
    assert rel_err(yr.cpu().numpy(), orr) <= 1e-12 and rel_err(yi.cpu().numpy(), oii) <= 1e-12
    import torch
    fr, fi = ctx.schro_res_f32(ctx.to_device(V, torch.float32), 0.0123, ctx.to_device(u, torch.float32),
                               ctx.to_device(v, torch.float32))
    assert rel_err(fr.cpu().numpy(), orr) <= 2e-5 and rel_err(fi.cpu().numpy(), oii) <= 2e-5


@pytest.mark.parametrize("precise", [True, False])
def test_neumann_schrodinger_steps(semlib, oracle, precise):
    """reflecting walls: two SDIRK4-3 steps of a packet aimed at the wall"""
    from schrodingersem_gb300 import capi
    from schrodingersem_gb300.meshgen import gaussian_packet
    co, el = structured(6, box=(-3.0, 3.0, -3.0, 3.0), jitter=0.1, seed=2)
    p = 6
    ctx = semlib.Context(p, coords=co, elements=el, neumann=True)
    om = oracle.Mesh(p, coords=co, elements=el, neumann=True)
    X, Y = om.node_coords()
    re, im = gaussian_packet(X, Y, (1.5, 0.0), 0.7, (4.0, 0.0))
    V = 0.5 * (X * X + Y * Y)
    dt, steps = 1e-2, 2
    pr, pi, ok = om.schrodinger("dirk4s3", re, im, V, (steps - 0.5) * dt, dt, 20 * om.dof(), 1e-12, n_steps=steps)
    assert ok
    if not precise:
        ctx.set_option(capi.OPT_SOLVE_PRECISION, capi.PREC_MIXED)
        ctx.set_option(capi.OPT_PRECOND, capi.PRECOND_FDM)
        ctx.set_option(capi.OPT_REFINE_TOL_SCALE, 0.1)
    gr, gi = re.copy(), im.copy()
    assert ctx.schrodinger("dirk4s3", gr, gi, V, (steps - 0.5) * dt, dt, 20 * ctx.dof(), 1e-12 if precise else 1e-10,
                           n_steps=steps)
    tol = 1e-9 if precise else 1e-8
    assert rel_err(gr, pr) <= tol and rel_err(gi, pi) <= tol
    # the boundary copies carry the wave (they are zero with Dirichlet masks)
    assert np.max(np.abs(gr[:, 0, :])) > 0


def test_dirichlet_data_matches_reference(semlib):
    fx = load_ref_fixture("bc_dirichlet")
    ctx = semlib.Context(6, folder=SMALL_MESH)
    u = np.zeros(ctx.shape)
    ok, it, _ = ctx.poisson_bc(u, fx["f"], fx["g"], ctx.dof(), float(fx["tol"]))
    assert ok and abs(it - int(fx["poisson_iters"])) <= 2
    assert rel_err(u, fx["poisson_u"]) <= 1e-10
    u = np.zeros(ctx.shape)
    ok, it, _ = ctx.helmholtz_bc(u, fx["c"], fx["f"], fx["g"], 10 * ctx.dof(), float(fx["tol"]))
    assert ok and abs(it - int(fx["helmholtz_iters"])) <= 0.02 * int(fx["helmholtz_iters"]) + 2
    assert rel_err(u, fx["helmholtz_u"]) <= 1e-9


@pytest.mark.parametrize("p", [3, 6])
def test_neumann_data_matches_oracle_and_manufactured(semlib, oracle, p):
    co, el = structured(8, box=(0.0, 1.0, 0.0, 1.0), jitter=0.15, seed=0)
    ctx = semlib.Context(p, coords=co, elements=el, corrected_metric=True, neumann=True)
    om = oracle.Mesh(p, coords=co, elements=el, ref_compat=False, neumann=True)
    X, Y = om.node_coords()
    g = dudn_sides(om, X, Y)
    c, f = np.ones(om.shape), harmonic(X, Y)
    uo, (ok_o, it_o, _) = om.helmholtz_bc(om.zeros(), c, f, g, 10 * om.dof(), 1e-13)
    u = np.zeros(ctx.shape)
    ok, it, _ = ctx.helmholtz_bc(u, c, f, np.ascontiguousarray(g), 10 * ctx.dof(), 1e-13)
    assert ok and ok_o and abs(it - it_o) <= 3
    assert rel_err(u, uo) <= 1e-10
    err = np.max(np.abs(u - harmonic(X, Y)))
    assert err < (2e-6 if p == 3 else 1e-11), err
    # device pointers give the same result
    import torch
    du = torch.zeros(ctx.shape, dtype=torch.float64, device="cuda")
    ok, it2, _ = ctx.helmholtz_bc(du, ctx.to_device(c), ctx.to_device(f),
                                  torch.as_tensor(np.ascontiguousarray(g), device="cuda"), 10 * ctx.dof(), 1e-13)
    assert ok and it2 == it and np.array_equal(du.cpu().numpy(), u)


def test_manufactured_dirichlet_poisson(semlib):
    """u = exp(x) sin(y) (harmonic) with its boundary values on a jittered
    unit square: the error falls from p = 3 to p = 6 as the discretisation's"""
    co, el = structured(8, box=(0.0, 1.0, 0.0, 1.0), jitter=0.15, seed=0)
    errs = []
    for p in (3, 6):
        ctx = semlib.Context(p, coords=co, elements=el, corrected_metric=True)
        X, Y = ctx.node_coords()
        u = np.zeros(ctx.shape)
        ok, _, _ = ctx.poisson_bc(u, np.zeros(ctx.shape), harmonic(X, Y), ctx.dof(), 1e-13)
        assert ok
        errs.append(np.max(np.abs(u - harmonic(X, Y))))
    assert errs[0] < 2e-6 and errs[1] < 1e-11, errs
