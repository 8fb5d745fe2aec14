"""Regenerate the committed fixtures under tests/golden/.

Run from the repository root in a container that has the reference mounted:
    python tests/golden/make_golden.py /path/to/reference
It copies the reference's sample mesh (meshes/small_mesh: 58 nodes, 45
unstructured quads, used by every reference integration test) and records
the known answers the reference's own tests assert, so that the tests never
read the reference at run time.
"""
import json
import os
import shutil
import sys

from scipy.special import i0

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    src = os.path.join(ref, "meshes", "small_mesh")
    dst = os.path.join(HERE, "small_mesh")
    os.makedirs(dst, exist_ok=True)
    for f in ("info.txt", "coordinates.txt", "elements.txt", "README.txt"):
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
    known = {
        # tests/gauss_lobatto.cpp:11-44: the p=9 rule integrates exp(sin(pi x))
        # over [-1,1] to within 1e-4 of 2*I0(1); p=10 does at least as well
        "lgl_integral_exact": float(2.0 * i0(1.0)),
        "lgl_integral_tol": 1e-4,
        # tests/derivative_matrix.cpp:4-35: D (p=8) is exact on
        # p(x) = -1 + 2x + 5x^2 - 3x^3 to 1e-10
        "cubic_coeffs": [-1.0, 2.0, 5.0, -3.0],
        "cubic_deriv_tol": 1e-10,
        # tests/glaplace.cpp:4-25: weak Laplacian of a constant on [-1,1]^2, p=5
        "glaplace_const_tol": 1e-10,
        # tests/pcg.cpp, tests/minres.cpp: 1-D FD problems, n = 20, tol 1e-5
        "fd_n": 20, "fd_tol": 1e-5, "fd_helmholtz_k": 2.0,
        # tests/poisson.cpp:11-34, tests/helmholtz.cpp:6-32 on small_mesh, p=6
        "poisson_p": 6, "poisson_tol": 1e-10,
        "helmholtz_p": 6, "helmholtz_tol": 1e-10, "helmholtz_c": -100.0 - 2.0 ** 0.5,
        # tests/schrodinger.cpp:18-124: p=3, V=0, psi0 = sin(pi x) sin(pi y),
        # T = 0.01, dt = T/10, tol 1e-8, max_iter = 20*dof
        "schro_p": 3, "schro_T": 0.01, "schro_steps": 10, "schro_tol": 1e-8,
        # mpi_tests/dot.cpp:9-33: dot(1, 1) equals the global DOF count
        "small_mesh_nodes": 58, "small_mesh_elements": 45,
    }
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(known, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
