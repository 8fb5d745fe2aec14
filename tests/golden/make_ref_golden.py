"""Generate the reference fixtures under tests/golden/ref/ from the reference
itself (its unmodified OpenMP headers built by ``oracle/ref``).

Run from the repository root where a reference checkout is available:
    python tests/golden/make_ref_golden.py <reference checkout>

Every fixture is computed with one OpenMP thread (the reference's dot
product is an OpenMP reduction whose summation order follows the thread
count; tests/tests.cpp:24 runs the reference's own suite on one thread too).
Inputs come from ``tests.util.det_field`` (integer arithmetic, the same on
every host) or are stored in the fixture.

Cases (``tests/util.py`` REF_MESHES names the synthetic meshes):
  small_p4, small_p8  the reference's sample mesh (meshes/small_mesh):
      quadrature, D, metrics, unmask, global_sum, mask, dot, gproj, the
      Poisson and Helmholtz galerkin operators and the Schroedinger Res and
      f operators
  small_p12  the same mesh at a degree whose quadrature comes from LAPACK
      (include/gauss_lobatto.hpp:60-113): quadrature, D, dot, gproj, the
      Poisson operator and Res
  jit8_p6   8x8 jittered quads on [-4,4]^2: the same operators, one MINRES
      solve on Res (include/minres.hpp), and three steps of each
      Schroedinger driver at MINRES tolerance 1e-12
  c1_p4     the Poisson configuration: 16x16 quads on [0,1]^2 jittered by
      0.15h (seed 0), p = 4, f = 2 pi^2 sin(pi x) sin(pi y), PCG to 1e-12
  reftests  the reference's own integration tests (tests/poisson.cpp,
      helmholtz.cpp, schrodinger.cpp) with their outputs and iteration counts
  bc_dirichlet  inhomogeneous Dirichlet data on the sample mesh, p = 6, by
      lifting composed of the reference's own gproj, galerkin operators,
      mask/unmask and PCG (Poisson) / MINRES (Helmholtz) to 1e-12
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from schrodingersem_gb300.meshgen import gaussian_packet, write_mesh_folder  # noqa: E402
from tests.util import REF_GOLDEN, SMALL_MESH, det_field, ref_mesh_arrays  # noqa: E402

ALPHA = 0.0123


def _ops(R, m, out, full=True):
    sh = m.shape
    u, v = det_field(sh, 1), det_field(sh, 2)
    V = det_field(sh, 3, -5.0, 5.0)
    c = det_field(sh, 4, 0.5, 2.0)
    out["x"], out["w"], out["D"] = m.x, m.w, m.D
    if full:
        out["unmask"] = m.unmask(u)
        out["global_sum"] = m.global_sum(u)
        out["mask"] = m.mask(u)
    out["dot_uv"] = np.array(m.dot(u, v))
    out["dot_11"] = np.array(m.dot(np.ones(sh), np.ones(sh)))
    out["dof"] = np.array(m.dof())
    out["gproj"] = m.gproj(u)
    out["laplace"] = m.apply_laplace(u)
    out["res_re"], out["res_im"] = m.schro_res(V, ALPHA, u, v)
    if full:
        out["helmholtz"] = m.apply_helmholtz(c, u)
        out["f_re"], out["f_im"] = m.schro_f(V, u, v)
    out["alpha"] = np.array(ALPHA)


def _metrics(m, out):
    out["J"], out["A"], out["B"], out["C"] = m.metrics()


def main(reference: str) -> None:
    os.environ["SEM_REFERENCE_DIR"] = reference
    from oracle import ref as R
    R.build()
    R.set_threads(1)
    os.makedirs(REF_GOLDEN, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="sem_ref_golden_")
    folders = {"small": SMALL_MESH}
    for name in ("jit8", "c1"):
        co, el = ref_mesh_arrays(name)
        folders[name] = os.path.join(tmp, name)
        write_mesh_folder(folders[name], co, el)

    def save(name, out):
        path = os.path.join(REF_GOLDEN, name + ".npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")

    for p in (4, 8, 12):
        m = R.Mesh(p, folders["small"])
        out = {"p": np.array(p)}
        _ops(R, m, out, full=p <= 8)
        if p <= 8:
            _metrics(m, out)
        save(f"small_p{p}", out)

    # jit8_p6: operators, one MINRES solve on Res, three steps of each driver
    p = 6
    m = R.Mesh(p, folders["jit8"])
    out = {"p": np.array(p)}
    _ops(R, m, out)
    X, Y = m.node_coords()
    Vh = 0.5 * (X * X + Y * Y)
    re0, im0 = gaussian_packet(X, Y, (-1.0, 0.0), 1.0, (2.0, 0.0))
    out["V_harm"], out["psi0_re"], out["psi0_im"] = Vh, re0, im0
    b_re, b_im = m.gproj(det_field(m.shape, 5)), m.gproj(det_field(m.shape, 6))
    out["mr_b_re"], out["mr_b_im"] = b_re, b_im
    mr_alpha, mr_tol, mr_maxit = 0.01, 1e-10, 10 * m.dof()
    xr, xi, (ok, it, res) = m.minres_res(Vh, mr_alpha, b_re, b_im, m.zeros(), m.zeros(), mr_maxit, mr_tol)
    assert ok
    out.update(mr_alpha=np.array(mr_alpha), mr_tol=np.array(mr_tol), mr_maxit=np.array(mr_maxit),
               mr_x_re=xr, mr_x_im=xi, mr_iters=np.array(it), mr_residual=np.array(res))
    dt, tol, steps = 1e-2, 1e-12, 3
    out.update(drv_dt=np.array(dt), drv_tol=np.array(tol), drv_steps=np.array(steps),
               drv_maxit=np.array(20 * m.dof()))
    for meth in ("bdf2", "dirk4s3", "dirk4s5"):
        pr, pi, ok, done, _ = m.schrodinger(meth, re0, im0, Vh, dt, 20 * m.dof(), tol, steps)
        assert ok and done == steps
        out[f"{meth}_re"], out[f"{meth}_im"] = pr, pi
    save("jit8_p6", out)

    # c1: the Poisson configuration at its full size
    p = 4
    m = R.Mesh(p, folders["c1"])
    X, Y = m.node_coords()
    f = 2.0 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y)
    u, (ok, it, res) = m.poisson(m.zeros(), f, m.dof(), 1e-12)
    assert ok
    exact = np.sin(np.pi * X) * np.sin(np.pi * Y)
    save("c1_p4", {"p": np.array(p), "f": f, "u": u, "n_iter": np.array(it), "residual": np.array(res),
                   "tol": np.array(1e-12), "max_iter": np.array(m.dof()), "X": X, "Y": Y,
                   "manufactured_err_max": np.array(np.max(np.abs(m.unmask(u) - exact)))})

    # the reference's own integration tests
    out = {}
    m = R.Mesh(6, folders["small"])
    X, Y = m.node_coords()
    F = X * X - Y * Y
    u, (ok, it, res) = m.poisson(m.zeros(), F, m.dof(), 1e-10)
    assert ok
    out.update(poisson_F=F, poisson_u=u, poisson_iters=np.array(it), poisson_residual=np.array(res))
    c = np.full(m.shape, -100.0 - np.sqrt(2.0))
    u, (ok, it, res) = m.helmholtz(m.zeros(), c, F, 10 * m.dof(), 1e-10)
    assert ok
    out.update(helmholtz_u=u, helmholtz_iters=np.array(it), helmholtz_residual=np.array(res))
    m = R.Mesh(3, folders["small"])
    X, Y = m.node_coords()
    re0 = np.sin(np.pi * X) * np.sin(np.pi * Y)
    out["schro_psi0_re"] = re0
    for meth in ("bdf2", "dirk4s3", "dirk4s5"):
        pr, pi, ok, done, _ = m.schrodinger(meth, re0, np.zeros_like(re0), np.zeros_like(re0), 1e-3,
                                            20 * m.dof(), 1e-8, 10)
        assert ok and done == 10
        out[f"schro_{meth}_re"], out[f"schro_{meth}_im"] = pr, pi
    save("reftests", out)

    # inhomogeneous Dirichlet data by lifting
    m = R.Mesh(6, folders["small"])
    X, Y = m.node_coords()
    g = np.exp(X) * np.sin(Y)
    f = np.cos(X) * Y
    c = 1.0 + 0.5 * np.sin(X)
    up, (okp, itp, rp) = m.dirichlet_bc(False, None, m.zeros(), f, g, m.dof(), 1e-12)
    uh, (okh, ith, rh) = m.dirichlet_bc(True, c, m.zeros(), f, g, 10 * m.dof(), 1e-12)
    assert okp and okh
    save("bc_dirichlet", {"p": np.array(6), "g": g, "f": f, "c": c, "poisson_u": up, "poisson_iters": np.array(itp),
                          "poisson_residual": np.array(rp), "helmholtz_u": uh, "helmholtz_iters": np.array(ith),
                          "helmholtz_residual": np.array(rh), "tol": np.array(1e-12)})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_golden.py <reference checkout>")
    main(sys.argv[1])
