"""The oracle restatement against the reference itself (CPU).

The fixtures under tests/golden/ref/ were produced by the reference's own
OpenMP implementation (its unmodified headers, built by oracle/ref against
this project's Armadillo/Boost/LAPACK shims) on one thread; see
tests/golden/make_ref_golden.py.  With one thread the oracle reproduces them
bit for bit at every degree whose quadrature comes from the reference's node
table (p <= 8): setup, gather-scatter, dot, every operator, MINRES and PCG
iterates and iteration counts, and whole Schroedinger trajectories.  For
p > 8 the reference takes its nodes from LAPACK's dsteqr plus two Newton
steps and the oracle from bisection plus the same Newton steps; the nodes
then differ in the last bit and results agree to 1e-14.

Where the reference can be built here (a checkout is present) the tests also
run it live on further meshes and run its own unit-test program against the
shims."""
import os
import subprocess

import numpy as np
import pytest

from tests.util import SMALL_MESH, det_field, load_ref_fixture, ref_mesh_arrays, rel_err, structured

OPS = ("unmask", "global_sum", "mask", "gproj", "laplace", "helmholtz", "res_re", "res_im", "f_re", "f_im")


@pytest.fixture()
def one_thread(oracle):
    n = oracle.get_threads()
    oracle.set_threads(1)
    yield oracle
    oracle.set_threads(n)


def _oracle_mesh(O, name, p):
    if name == "small":
        return O.Mesh(p, folder=SMALL_MESH)
    co, el = ref_mesh_arrays(name)
    return O.Mesh(p, coords=co, elements=el)


def _ops(om, fx):
    sh = om.shape
    u, v = det_field(sh, 1), det_field(sh, 2)
    V = det_field(sh, 3, -5.0, 5.0)
    c = det_field(sh, 4, 0.5, 2.0)
    alpha = float(fx["alpha"])
    got = {"unmask": om.unmask(u), "global_sum": om.global_sum(u), "mask": om.mask(u), "gproj": om.gproj(u),
           "laplace": om.apply_laplace(u), "helmholtz": om.apply_helmholtz(c, u)}
    got["res_re"], got["res_im"] = om.schro_res(V, alpha, u, v)
    got["f_re"], got["f_im"] = om.schro_f(V, u, v)
    return got, om.dot(u, v)


@pytest.mark.parametrize("case,mesh,p", [("small_p4", "small", 4), ("small_p8", "small", 8),
                                         ("small_p12", "small", 12), ("jit8_p6", "jit8", 6)])
def test_oracle_operators_match_reference(one_thread, case, mesh, p):
    fx = load_ref_fixture(case)
    om = _oracle_mesh(one_thread, mesh, p)
    exact = p <= 8
    assert om.dof() == int(fx["dof"])
    got, dot_uv = _ops(om, fx)
    for k, want in (("x", om.x), ("w", om.w), ("D", om.D)):
        if exact:
            assert np.array_equal(fx[k], want), k
        else:
            assert np.max(np.abs(fx[k] - want)) <= 1e-14 * max(1.0, np.max(np.abs(fx[k]))), k
    if "J" in fx:
        for k, want in (("J", om.J), ("A", om.A), ("B", om.B), ("C", om.C)):
            assert np.array_equal(fx[k], want), k
    for k in OPS:
        if k not in fx:
            continue
        if exact:
            assert np.array_equal(got[k], fx[k]), k
        else:
            assert rel_err(got[k], fx[k]) <= 1e-14, k
    if exact:
        assert dot_uv == float(fx["dot_uv"])
    else:
        assert abs(dot_uv - float(fx["dot_uv"])) <= 1e-14 * abs(float(fx["dot_uv"]))
    assert om.dot(np.ones(om.shape), np.ones(om.shape)) == float(fx["dot_11"]) == om.dof()


def test_oracle_minres_matches_reference(one_thread):
    """The reference's MINRES (include/minres.hpp:19-107) on Res: the same
    iterates, residual estimate and iteration count."""
    O = one_thread
    fx = load_ref_fixture("jit8_p6")
    om = _oracle_mesh(O, "jit8", 6)
    V, alpha = fx["V_harm"], float(fx["mr_alpha"])
    n = om.n_el * om.N * om.N

    def apply(q):
        a, b = om.schro_res(V, alpha, q[:n].reshape(om.shape), q[n:].reshape(om.shape))
        return np.concatenate([a.ravel(), b.ravel()])

    def dot(a, b):
        return om.dot(a[:n].reshape(om.shape), b[:n].reshape(om.shape)) + \
            om.dot(a[n:].reshape(om.shape), b[n:].reshape(om.shape))

    b = np.concatenate([fx["mr_b_re"].ravel(), fx["mr_b_im"].ravel()])
    x, (ok, it, res) = O.krylov("minres", apply, b, np.zeros(2 * n), int(fx["mr_maxit"]), float(fx["mr_tol"]),
                                dot=dot)
    assert ok
    assert it == int(fx["mr_iters"])
    assert res == float(fx["mr_residual"])
    assert np.array_equal(x[:n].reshape(om.shape), fx["mr_x_re"])
    assert np.array_equal(x[n:].reshape(om.shape), fx["mr_x_im"])


@pytest.mark.parametrize("method", ["bdf2", "dirk4s3", "dirk4s5"])
def test_oracle_drivers_match_reference(one_thread, method):
    fx = load_ref_fixture("jit8_p6")
    om = _oracle_mesh(one_thread, "jit8", 6)
    dt, steps = float(fx["drv_dt"]), int(fx["drv_steps"])
    pr, pi, ok = om.schrodinger(method, fx["psi0_re"], fx["psi0_im"], fx["V_harm"], dt * (steps + 1), dt,
                                int(fx["drv_maxit"]), float(fx["drv_tol"]), n_steps=steps)
    assert ok
    assert np.array_equal(pr, fx[f"{method}_re"]) and np.array_equal(pi, fx[f"{method}_im"])


def test_oracle_poisson_c1_matches_reference(one_thread):
    """The Poisson configuration (16x16, jitter 0.15, seed 0, p = 4, PCG 1e-12)."""
    fx = load_ref_fixture("c1_p4")
    om = _oracle_mesh(one_thread, "c1", 4)
    u, (ok, it, res) = om.poisson(om.zeros(), fx["f"], int(fx["max_iter"]), float(fx["tol"]))
    assert ok and it == int(fx["n_iter"]) and res == float(fx["residual"])
    assert np.array_equal(u, fx["u"])
    # manufactured solution u = sin(pi x) sin(pi y): the reference's metric
    # C = (Yxi[i]^2 + Xxi[j]^2)/J (include/Quad.hpp:53) is not the metric of
    # a jittered quad, so its solution stays ~1e-3 away; with the corrected
    # metric the same solve is within 4e-9 and the error falls spectrally in p
    assert 5e-4 < float(fx["manufactured_err_max"]) < 2e-3
    co, el = ref_mesh_arrays("c1")
    errs = []
    for p in (2, 4, 6):
        cm = one_thread.Mesh(p, coords=co, elements=el, ref_compat=False)
        X, Y = cm.node_coords()
        f = 2.0 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
        uc, (ok, _, _) = cm.poisson(cm.zeros(), f, cm.dof(), 1e-13)
        assert ok
        errs.append(np.max(np.abs(cm.unmask(uc) - np.sin(np.pi * X) * np.sin(np.pi * Y))))
    assert errs[1] < 1e-8 and errs[2] < 1e-11 and errs[0] > 100 * errs[1] > 1e4 * errs[2]


def test_oracle_reference_integration_tests(one_thread):
    """tests/poisson.cpp, helmholtz.cpp, schrodinger.cpp of the reference."""
    O = one_thread
    fx = load_ref_fixture("reftests")
    om = O.Mesh(6, folder=SMALL_MESH)
    u, (ok, it, res) = om.poisson(om.zeros(), fx["poisson_F"], om.dof(), 1e-10)
    assert ok and it == int(fx["poisson_iters"]) and np.array_equal(u, fx["poisson_u"])
    c = np.full(om.shape, -100.0 - np.sqrt(2.0))
    u, (ok, it, res) = om.helmholtz(om.zeros(), c, fx["poisson_F"], 10 * om.dof(), 1e-10)
    assert ok and it == int(fx["helmholtz_iters"]) and np.array_equal(u, fx["helmholtz_u"])
    om = O.Mesh(3, folder=SMALL_MESH)
    re0 = fx["schro_psi0_re"]
    z = np.zeros_like(re0)
    for meth in ("bdf2", "dirk4s3", "dirk4s5"):
        pr, pi, ok = om.schrodinger(meth, re0, z, z, 0.0105, 1e-3, 20 * om.dof(), 1e-8, n_steps=10)
        assert ok
        assert np.array_equal(pr, fx[f"schro_{meth}_re"]) and np.array_equal(pi, fx[f"schro_{meth}_im"]), meth


# ---------------------------------------------------------------- live reference
def _ref():
    try:
        from oracle import ref as R
        R.lib()
        return R
    except Exception as e:  # no checkout and nothing staged on this host
        pytest.skip(f"reference build unavailable: {e}")


@pytest.mark.parametrize("p", [1, 2, 5, 7, 8])
def test_live_reference_shuffled_mesh(one_thread, tmp_path, p):
    """Elements in a shuffled order with rotated corner lists (every edge
    orientation case of include/load_mesh.hpp:146-203): oracle == reference."""
    from schrodingersem_gb300.meshgen import write_mesh_folder
    R = _ref()
    R.set_threads(1)
    co, el = structured(4, box=(-1.0, 1.5, -2.0, 0.5), jitter=0.2, seed=40 + p)
    rng = np.random.default_rng(p)
    el = el[rng.permutation(len(el))]
    el = np.stack([np.roll(r, int(k)) for r, k in zip(el, rng.integers(0, 4, len(el)))]).astype(np.int32)
    write_mesh_folder(str(tmp_path), co, el)
    rm = R.Mesh(p, str(tmp_path))
    om = one_thread.Mesh(p, coords=co, elements=el)
    sh = om.shape
    u, v = det_field(sh, 11), det_field(sh, 12)
    V = det_field(sh, 13, 0.0, 3.0)
    assert np.array_equal(rm.metrics()[3], om.C)
    for name in ("unmask", "global_sum", "mask", "gproj", "apply_laplace"):
        assert np.array_equal(getattr(rm, name)(u), getattr(om, name)(u)), name
    assert rm.dot(u, v) == om.dot(u, v)
    a, b = rm.schro_res(V, 0.02, u, v), om.schro_res(V, 0.02, u, v)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    X, Y = rm.node_coords()
    F = np.cos(X) * Y
    ur, rr = rm.poisson(rm.zeros(), F, rm.dof(), 1e-11)
    uo, ro = om.poisson(om.zeros(), F, om.dof(), 1e-11)
    assert rr == ro and np.array_equal(ur, uo)
    re0, im0 = np.exp(-(X * X + Y * Y)), 0.3 * X * np.exp(-(X * X + Y * Y))
    a = rm.schrodinger("dirk4s3", re0, im0, V, 5e-3, 20 * rm.dof(), 1e-11, 2)
    b = om.schrodinger("dirk4s3", re0, im0, V, 0.0125, 5e-3, 20 * om.dof(), 1e-11, n_steps=2)
    assert a[2] and b[2] and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_reference_unit_suite_passes_against_shims(tmp_path):
    """The reference's own unit-test program (tests/*.cpp: quadrature
    integral vs 2 I0(1), D exact on a cubic, glaplace(1) = 0, FD PCG and
    MINRES residuals, wrapper algebra, and convergence of the Poisson,
    Helmholtz and three Schroedinger drivers on the sample mesh), compiled
    unmodified against this project's shims, reports that all tests pass."""
    R = _ref()
    src = R.checkout()
    if src is None:
        pytest.skip("no reference checkout on this host")
    here = os.path.join(os.path.dirname(R.__file__), "ref")
    subprocess.run(["make", "-s", "-C", here, "ref-tests", f"REFERENCE={src}"], check=True,
                   stdout=subprocess.DEVNULL)
    exe = os.path.join(os.path.dirname(R.__file__), "_ref", "tests", "ref_tests.out")
    run = tmp_path / "tests"
    run.mkdir()
    meshes = tmp_path / "meshes"
    meshes.mkdir()
    os.symlink(SMALL_MESH, meshes / "small_mesh")
    env = dict(os.environ)
    lp = R.lapack_path()
    if lp:
        env["SEM_REF_LAPACK"] = lp
    r = subprocess.run([exe], cwd=str(run), env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "all tests passed!" in r.stdout, r.stdout[-2000:]
