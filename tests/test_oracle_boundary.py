"""Boundary data beyond the reference's homogeneous Dirichlet masks (CPU).

The reference zeroes every boundary copy (include/mask_side.hpp:28-30 says
the boundary branch "needs to be modified for Neumann").  Two extensions:
  * inhomogeneous Dirichlet data by lifting: u_D = g on the boundary, solve
    the masked system with b = gproj(f) - A u_D, u = u0 + u_D.  Composed of
    the reference's own primitives (its gproj, galerkin operators, masks and
    PCG/MINRES) it gives the fixture tests/golden/ref/bc_dirichlet.npz, which
    the oracle's composition reproduces bit for bit;
  * natural (Neumann) boundaries: boundary edges and corners are ordinary
    degrees of freedom, and du/dn = g enters as the boundary integral of the
    weak form.
Both are checked against manufactured solutions on jittered meshes (with
the corrected metric the errors fall spectrally in p)."""
import numpy as np
import pytest

from tests.util import SMALL_MESH, load_ref_fixture, structured


@pytest.fixture()
def one_thread(oracle):
    n = oracle.get_threads()
    oracle.set_threads(1)
    yield oracle
    oracle.set_threads(n)


def harmonic(X, Y):
    return np.exp(X) * np.sin(Y)  # -lap u = 0


def dudn_sides(om, X, Y):
    """outward normal derivative of exp(x) sin(y) at every element side node,
    shape (E, 4, N) (library sides 0: j = 0, 1: i = N-1, 2: j = N-1, 3: i = 0)"""
    E, N = om.n_el, om.N
    g = np.zeros((E, 4, N))
    ca, cb = (0, 1, 3, 0), (1, 2, 2, 3)
    for e in range(E):
        for s in range(4):
            jj, ii = om._side_index(s)
            x, y = X[e, jj, ii], Y[e, jj, ii]
            tx, ty = om.xs[e, cb[s]] - om.xs[e, ca[s]], om.ys[e, cb[s]] - om.ys[e, ca[s]]
            nx, ny = (ty, -tx) if s in (0, 1) else (-ty, tx)  # counter-clockwise elements
            L = np.hypot(nx, ny)
            g[e, s] = (np.exp(x) * np.sin(y) * nx + np.exp(x) * np.cos(y) * ny) / L
    return g


def test_dirichlet_lifting_matches_reference(one_thread):
    fx = load_ref_fixture("bc_dirichlet")
    om = one_thread.Mesh(6, folder=SMALL_MESH)
    u, (ok, it, res) = om.poisson_bc(om.zeros(), fx["f"], fx["g"], om.dof(), float(fx["tol"]))
    assert ok and it == int(fx["poisson_iters"]) and res == float(fx["poisson_residual"])
    assert np.array_equal(u, fx["poisson_u"])
    u, (ok, it, res) = om.helmholtz_bc(om.zeros(), fx["c"], fx["f"], fx["g"], 10 * om.dof(), float(fx["tol"]))
    assert ok and it == int(fx["helmholtz_iters"]) and res == float(fx["helmholtz_residual"])
    assert np.array_equal(u, fx["helmholtz_u"])


def test_manufactured_dirichlet_and_neumann_converge_spectrally(oracle):
    co, el = structured(8, box=(0.0, 1.0, 0.0, 1.0), jitter=0.15, seed=0)
    errs_d, errs_n = [], []
    for p in (2, 4, 6):
        om = oracle.Mesh(p, coords=co, elements=el, ref_compat=False)
        X, Y = om.node_coords()
        u, (ok, _, _) = om.poisson_bc(om.zeros(), np.zeros(om.shape), harmonic(X, Y), om.dof(), 1e-13)
        assert ok
        errs_d.append(np.max(np.abs(u - harmonic(X, Y))))
        on = oracle.Mesh(p, coords=co, elements=el, ref_compat=False, neumann=True)
        # -lap u + u = u for the harmonic u: Helmholtz with c = 1, f = u
        u, (ok, _, _) = on.helmholtz_bc(on.zeros(), np.ones(on.shape), harmonic(X, Y), dudn_sides(on, X, Y),
                                        10 * on.dof(), 1e-13)
        assert ok
        errs_n.append(np.max(np.abs(u - harmonic(X, Y))))
    for e in (errs_d, errs_n):
        assert e[0] < 1e-4 and e[1] < 2e-9 and e[2] < 2e-12, e


def test_neumann_mesh_keeps_boundary_dofs(oracle):
    om = oracle.Mesh(4, folder=SMALL_MESH, neumann=True)
    one = np.ones(om.shape)
    assert om.dot(one, one) == om.dof()
    # the mass of the constant over every degree of freedom is the domain's
    # area (GLL quadrature of a bilinear Jacobian is exact); the Dirichlet
    # mesh drops the boundary rows
    od = oracle.Mesh(4, folder=SMALL_MESH)
    area = float(np.sum(od.J * od.w[None, :, None] * od.w[None, None, :]))
    assert abs(om.dot(om.gproj(one), one) - area) <= 1e-12 * area
    assert od.dot(od.gproj(one), one) < area
    # homogeneous Neumann: the Laplacian of a constant is zero in every row
    assert np.max(np.abs(om.apply_laplace(one))) < 1e-11
