"""Pin the CPU oracle against every known-answer test the reference's own
test-suite holds for the hot path (tests/*.cpp, mpi_tests/dot.cpp), on the
reference's sample mesh (tests/golden/small_mesh)."""
import numpy as np
import pytest

from tests.util import SMALL_MESH, rel_err, structured


def test_gauss_lobatto_integral(oracle, known):
    # tests/gauss_lobatto.cpp:11-44 (p=9 exercises the eigenvalue path)
    f = lambda x: np.exp(np.sin(np.pi * x))  # noqa: E731
    x9, w9 = oracle.gauss_lobatto(9)
    x10, w10 = oracle.gauss_lobatto(10)
    e1 = abs(np.sum(f(x9) * w9) - known["lgl_integral_exact"])
    e2 = abs(np.sum(f(x10) * w10) - known["lgl_integral_exact"])
    assert e1 <= known["lgl_integral_tol"]
    assert e2 <= e1


@pytest.mark.parametrize("p", range(1, 17))
def test_gauss_lobatto_nodes(oracle, p):
    x, w = oracle.gauss_lobatto(p)
    assert x[0] == -1 and x[-1] == 1 and np.all(np.diff(x) > 0)
    assert abs(w.sum() - 2.0) < 1e-13
    # symmetric and exact for polynomials of degree 2p-1
    assert np.allclose(x, -x[::-1], atol=1e-14)
    for k in range(0, 2 * p):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.sum(w * x ** k) - exact) < 1e-12
    if p >= 2:  # interior nodes are the roots of P_p'
        c = np.zeros(p + 1)
        c[p] = 1
        r = np.sort(np.polynomial.legendre.legroots(np.polynomial.legendre.legder(c)))
        assert np.max(abs(x[1:-1] - r)) < 1e-13


def test_derivative_matrix_cubic(oracle, known):
    # tests/derivative_matrix.cpp:14-35
    x, _ = oracle.gauss_lobatto(8)
    D = oracle.derivative_matrix(x)
    a0, a1, a2, a3 = known["cubic_coeffs"]
    y = a0 + a1 * x + a2 * x ** 2 + a3 * x ** 3
    dy = a1 + 2 * a2 * x + 3 * a3 * x ** 2
    assert np.max(abs(D @ y - dy)) < known["cubic_deriv_tol"]


def test_glaplace_constant(oracle, known):
    # tests/glaplace.cpp:4-25: one reference square element, p = 5
    m = oracle.Mesh(5, coords=[[-1, -1], [1, -1], [1, 1], [-1, 1]], elements=[[0, 1, 2, 3]])
    out = m.glaplace(0, np.ones((m.N, m.N)))
    assert np.max(abs(out)) < known["glaplace_const_tol"]


def _fd(n, k):
    x = np.linspace(-1, 1, n)
    h = x[1] - x[0]

    def L(u):  # arma::conv(u, {-1,2,-1}/h^2, "same") - k u
        return np.convolve(u, np.array([-1.0, 2.0, -1.0]) / h ** 2, mode="same") - k * u
    return x, L


def test_pcg_fd_poisson(oracle, known):
    # tests/pcg.cpp:5-29
    n, tol = known["fd_n"], known["fd_tol"]
    x, L = _fd(n, 0.0)
    f = x * x
    u, r = oracle.krylov("pcg", L, f, np.zeros(n), n, tol)
    assert np.linalg.norm(L(u) - f) <= tol * np.linalg.norm(f)


def test_minres_fd_helmholtz(oracle, known):
    # tests/minres.cpp:5-30 (indefinite)
    n, tol = known["fd_n"], known["fd_tol"]
    x, L = _fd(n, known["fd_helmholtz_k"])
    f = x * x
    u, r = oracle.krylov("minres", L, f, np.zeros(n), n, tol)
    assert np.linalg.norm(L(u) - f) <= tol * np.linalg.norm(f)


def test_small_mesh_topology(oracle, known):
    m = oracle.Mesh(3, folder=SMALL_MESH)
    assert (m.n_nodes, m.n_el) == (known["small_mesh_nodes"], known["small_mesh_elements"])
    # every edge has one or two elements; Euler: V - E_edges + F = 1 for a disc
    assert m.n_nodes - m.n_edges + m.n_el == 1
    val = np.diff(m.node_ptr)
    assert val.sum() == 4 * m.n_el
    # boundary edges form one closed loop: as many boundary nodes as edges
    assert (m.edge_type == 1).sum() == (m.node_type == 1).sum()


@pytest.mark.parametrize("p", [1, 3, 6])
def test_dot_ones_is_dof(oracle, p):
    # mpi_tests/dot.cpp:9-33
    m = oracle.Mesh(p, folder=SMALL_MESH)
    one = np.ones(m.shape)
    assert m.dot(one, one) == m.dof()


def test_mask_unmask_invariants(oracle):
    m = oracle.Mesh(4, folder=SMALL_MESH)
    rng = np.random.default_rng(0)
    a = rng.standard_normal(m.shape)
    b = m.mask(m.global_sum(a))
    # unmask(mask(x)) restores every shared copy; masking again is idempotent
    assert np.array_equal(m.mask(m.unmask(b)), b)
    assert np.array_equal(m.mask(b), b)
    # dot is invariant under unmask for masked vectors
    assert abs(m.dot(b, b) - m.dot(m.unmask(b), m.unmask(b))) <= 1e-12 * m.dot(b, b)


def test_operator_symmetry(oracle):
    # the Galerkin operators are symmetric in the unique-DOF inner product
    m = oracle.Mesh(5, folder=SMALL_MESH)
    rng = np.random.default_rng(1)
    u = m.mask(rng.standard_normal(m.shape))
    v = m.mask(rng.standard_normal(m.shape))
    Au, Av = m.apply_laplace(u), m.apply_laplace(v)
    assert abs(m.dot(Au, v) - m.dot(u, Av)) < 1e-11 * abs(m.dot(Au, v))
    V = rng.standard_normal(m.shape)
    r1 = m.schro_res(V, 0.3, u, v)
    r2 = m.schro_res(V, 0.3, v, u)
    # Res = [M, aL; aL, -M] is symmetric: <Res(u,v), (v,u)> = <(u,v), Res(v,u)>
    lhs = m.dot(r1[0], v) + m.dot(r1[1], u)
    rhs = m.dot(u, r2[0]) + m.dot(v, r2[1])
    assert abs(lhs - rhs) < 1e-11 * max(1.0, abs(lhs))


def test_poisson_converges(oracle, known):
    # tests/poisson.cpp:11-34
    m = oracle.Mesh(known["poisson_p"], folder=SMALL_MESH)
    X, Y = m.node_coords()
    u, (ok, it, res) = m.poisson(m.zeros(), X * X - Y * Y, m.dof(), known["poisson_tol"])
    assert ok and it < m.dof()


def test_helmholtz_converges(oracle, known):
    # tests/helmholtz.cpp:6-32
    m = oracle.Mesh(known["helmholtz_p"], folder=SMALL_MESH)
    X, Y = m.node_coords()
    c = np.full(m.shape, known["helmholtz_c"])
    u, (ok, it, res) = m.helmholtz(m.zeros(), c, X * X - Y * Y, 10 * m.dof(), known["helmholtz_tol"])
    assert ok


@pytest.mark.parametrize("method", ["bdf2", "dirk4s3", "dirk4s5"])
def test_schrodinger_converges(oracle, known, method):
    # tests/schrodinger.cpp:18-124
    m = oracle.Mesh(known["schro_p"], folder=SMALL_MESH)
    X, Y = m.node_coords()
    rec = []
    pr, pi, ok = m.schrodinger(method, np.sin(np.pi * X) * np.sin(np.pi * Y), m.zeros(), m.zeros(),
                               known["schro_T"], known["schro_T"] / known["schro_steps"], 20 * m.dof(),
                               known["schro_tol"], record=rec)
    assert ok and len(rec) == known["schro_steps"]


def test_manufactured_poisson_converges_spectrally(oracle):
    # -lap u = 2 pi^2 sin(pi x) sin(pi y) on a jittered mesh of [0,1]^2; with
    # the corrected metric the error falls fast with p
    errs = []
    for p in (2, 4, 6):
        co, el = structured(4, jitter=0.15, seed=0)
        m = oracle.Mesh(p, coords=co, elements=el, ref_compat=False)
        X, Y = m.node_coords()
        f = 2 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
        u, (ok, it, res) = m.poisson(m.zeros(), f, 10 * m.dof(), 1e-13)
        assert ok
        errs.append(rel_err(m.unmask(u), np.sin(np.pi * X) * np.sin(np.pi * Y)))
    assert errs[1] < errs[0] / 20 and errs[2] < errs[1] / 20


def test_reference_metric_formula_differs_on_jittered_quads(oracle):
    # include/Quad.hpp:53 uses Y_xi[i] where Y_xi[j] is the derivative at the
    # node; both agree on parallelograms and differ on jittered quads
    co, el = structured(3, jitter=0.2, seed=3)
    a = oracle.Mesh(3, coords=co, elements=el, ref_compat=True)
    b = oracle.Mesh(3, coords=co, elements=el, ref_compat=False)
    assert np.array_equal(a.A, b.A) and np.array_equal(a.B, b.B) and np.array_equal(a.J, b.J)
    assert not np.allclose(a.C, b.C)
    co, el = structured(3, jitter=0.0)
    a = oracle.Mesh(3, coords=co, elements=el, ref_compat=True)
    b = oracle.Mesh(3, coords=co, elements=el, ref_compat=False)
    assert np.allclose(a.C, b.C, rtol=1e-15, atol=0)
