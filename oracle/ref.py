"""ctypes loader for the reference's own OpenMP implementation.

TEST INFRASTRUCTURE ONLY.  ``oracle/_ref/libsemref.so`` is the reference
(header-only C++20, ``include/openmp_impl/*``) compiled unmodified against
this project's shims (``oracle/ref/shim``: an Armadillo subset and Boost.Math
Legendre/Bessel; LAPACK ``dsteqr`` forwarded to SciPy's bundled OpenBLAS).
It pins the oracle restatement, generates the golden fixtures under
``tests/golden/ref/`` and is the timed CPU baseline.  Only ``tests/``,
``bench.py``'s reference arm and CPU-baseline leg, and the fixture script may
import this module.

Building: ``build()`` stages the reference's headers from a reference
checkout (``SEM_REFERENCE_DIR``, default the checkout this container mounts)
into ``oracle/_ref/include`` and compiles them with ``oracle/ref/Makefile``.
Where no checkout exists (the GPU host) it compiles the headers already
staged there.  Fields use the oracle's layout: (E, N, N) float64 arrays
indexed [e, j, i], i.e. the column-major memory of the reference's
``std::vector<arma::Mat>``.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_OUT = os.path.join(_HERE, "_ref")
_LIB_PATH = os.path.join(_OUT, "libsemref.so")
_MAKE_DIR = os.path.join(_HERE, "ref")
_DEFAULT_CHECKOUT = "/root/reference"
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

METHODS = {"bdf2": 0, "dirk4s3": 1, "dirk4s5": 2}


class Unavailable(RuntimeError):
    """The reference build cannot be made on this host."""


def checkout() -> str | None:
    d = os.environ.get("SEM_REFERENCE_DIR", _DEFAULT_CHECKOUT)
    return d if os.path.isfile(os.path.join(d, "include", "minres.hpp")) else None


def staged() -> bool:
    return os.path.isfile(os.path.join(_OUT, "include", "minres.hpp"))


def lapack_path() -> str | None:
    """SciPy's bundled OpenBLAS (exports scipy_dsteqr_), if present."""
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(os.path.dirname(scipy.__file__))
    for pat in ("scipy.libs/libscipy_openblas*.so*", "scipy/.libs/libscipy_openblas*.so*",
                "scipy.libs/libopenblas*.so*", "scipy/.libs/libopenblas*.so*"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


def build(force: bool = False) -> str:
    """Stage the reference headers (when a checkout is present) and compile."""
    src = checkout()
    if src is not None:
        subprocess.run(["make", "-s", "-C", _MAKE_DIR, "stage", f"REFERENCE={src}"], check=True,
                       stdout=subprocess.DEVNULL)
    if not staged():
        raise Unavailable("the reference's headers are neither checked out nor staged in oracle/_ref/include")
    args = ["make", "-s", "-C", _MAKE_DIR]
    if force:
        args.insert(1, "-B")
    subprocess.run(args, check=True)
    return _LIB_PATH


def available() -> bool:
    try:
        lib()
        return True
    except Exception:
        return False


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.ref_last_error.restype = C.c_char_p
        L.ref_set_lapack.argtypes = [C.c_char_p]
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_get_threads.restype = C.c_int
        L.ref_mesh_load.argtypes = [C.c_int, C.c_char_p]
        L.ref_mesh_load.restype = C.c_void_p
        L.ref_mesh_free.argtypes = [C.c_void_p]
        L.ref_mesh_info.argtypes = [C.c_void_p] + [_ip] * 5
        L.ref_quadrature.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.ref_metrics.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.ref_node_coords.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_edges.argtypes = [C.c_void_p, _ip]
        L.ref_node_count_links.argtypes = [C.c_void_p]
        L.ref_node_count_links.restype = C.c_int
        L.ref_nodes.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _ip]
        for fn in ("ref_unmask", "ref_global_sum", "ref_mask"):
            getattr(L, fn).argtypes = [C.c_void_p, _dp]
        L.ref_dot.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_dot.restype = C.c_double
        L.ref_glaplace.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_gproj.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_laplace_op.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_helmholtz_op.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.ref_schro_res.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _dp, _dp, _dp]
        L.ref_schro_f.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.ref_poisson.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, _ip, _dp]
        L.ref_helmholtz.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_double, _ip, _dp]
        L.ref_minres_res.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _dp, _dp, _dp, C.c_int, C.c_double,
                                     _ip, _dp]
        L.ref_pcg_laplace.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, _ip, _dp]
        L.ref_minres_helmholtz.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_double, _ip, _dp]
        L.ref_schrodinger.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_double, C.c_int, C.c_double,
                                      C.c_int, C.c_int, C.c_double, _dp, _ip]
        lp = lapack_path()
        if lp is not None:
            L.ref_set_lapack(lp.encode())
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _f(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n: int) -> None:
    lib().ref_set_threads(int(n))


def get_threads() -> int:
    return int(lib().ref_get_threads())


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise RuntimeError(f"reference {what}: {lib().ref_last_error().decode(errors='replace')}")
    return rc


class Mesh:
    """``load_mesh<schro_omp::Mesh<double>>(p, folder)`` + ``compute_metrics()``
    of the reference (include/load_mesh.hpp:76-209, include/openmp_impl/
    Mesh.hpp:70-75)."""

    def __init__(self, p: int, folder: str):
        L = lib()
        h = L.ref_mesh_load(int(p), folder.encode())
        if not h:
            raise ValueError(f"reference load_mesh: {L.ref_last_error().decode(errors='replace')}")
        self._h = h
        v = [C.c_int() for _ in range(5)]
        L.ref_mesh_info(h, *[C.byref(t) for t in v])
        self.N, self.n_el, self.n_nodes, self.n_edges, self._dof = (int(t.value) for t in v)
        self.p = int(p)
        N = self.N
        self.x, self.w, Dc = np.zeros(N), np.zeros(N), np.zeros(N * N)
        L.ref_quadrature(h, _p(self.x), _p(self.w), _p(Dc))
        self.D = Dc.reshape(N, N).T.copy()  # column-major -> [i, j]

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().ref_mesh_free(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def shape(self):
        return (self.n_el, self.N, self.N)

    def zeros(self):
        return np.zeros(self.shape)

    def dof(self) -> int:
        return self._dof

    def metrics(self):
        J, A, B, Cm = (self.zeros() for _ in range(4))
        lib().ref_metrics(self._h, _p(J), _p(A), _p(B), _p(Cm))
        return J, A, B, Cm

    def node_coords(self):
        X, Y = self.zeros(), self.zeros()
        lib().ref_node_coords(self._h, _p(X), _p(Y))
        return X, Y

    def edges(self) -> np.ndarray:
        """(n_edges, 7) int: elements[0..1], element_sides[0..1], startIter,
        deltaIter, boundary flag, in the mesh's edge order."""
        out = np.zeros(7 * self.n_edges, dtype=np.int32)
        lib().ref_edges(self._h, out.ctypes.data_as(_ip))
        return out.reshape(-1, 7)

    def nodes(self):
        n = lib().ref_node_count_links(self._h)
        t = np.zeros(self.n_nodes, dtype=np.int32)
        ptr = np.zeros(self.n_nodes + 1, dtype=np.int32)
        el, ii, jj = (np.zeros(n, dtype=np.int32) for _ in range(3))
        lib().ref_nodes(self._h, *(a.ctypes.data_as(_ip) for a in (t, ptr, el, ii, jj)))
        return t, ptr, el, ii, jj

    def _inplace(self, fn, a):
        a = _f(a).copy()
        fn(self._h, _p(a))
        return a

    def unmask(self, a):
        return self._inplace(lib().ref_unmask, a)

    def global_sum(self, a):
        return self._inplace(lib().ref_global_sum, a)

    def mask(self, a):
        return self._inplace(lib().ref_mask, a)

    def dot(self, a, b) -> float:
        return float(lib().ref_dot(self._h, _p(_f(a)), _p(_f(b))))

    def glaplace_all(self, u):
        out = self.zeros()
        lib().ref_glaplace(self._h, _p(_f(u)), _p(out))
        return out

    def gproj(self, u):
        out = self.zeros()
        lib().ref_gproj(self._h, _p(_f(u)), _p(out))
        return out

    def apply_laplace(self, u):
        out = self.zeros()
        lib().ref_laplace_op(self._h, _p(_f(u)), _p(out))
        return out

    def apply_helmholtz(self, c, u):
        out = self.zeros()
        lib().ref_helmholtz_op(self._h, _p(_f(c)), _p(_f(u)), _p(out))
        return out

    def schro_res(self, V, alpha, q_re, q_im):
        y0, y1 = self.zeros(), self.zeros()
        lib().ref_schro_res(self._h, _p(_f(V)), float(alpha), _p(_f(q_re)), _p(_f(q_im)), _p(y0), _p(y1))
        return y0, y1

    def schro_f(self, V, q_re, q_im):
        y0, y1 = self.zeros(), self.zeros()
        lib().ref_schro_f(self._h, _p(_f(V)), _p(_f(q_re)), _p(_f(q_im)), _p(y0), _p(y1))
        return y0, y1

    def poisson(self, u, f, max_iter, tol):
        u = _f(u).copy()
        it, res = C.c_int(), C.c_double()
        ok = _check(lib().ref_poisson(self._h, _p(u), _p(_f(f)), int(max_iter), float(tol), C.byref(it),
                                      C.byref(res)), "poisson")
        return u, (bool(ok), int(it.value), float(res.value))

    def helmholtz(self, u, c, f, max_iter, tol):
        u = _f(u).copy()
        it, res = C.c_int(), C.c_double()
        ok = _check(lib().ref_helmholtz(self._h, _p(u), _p(_f(c)), _p(_f(f)), int(max_iter), float(tol),
                                        C.byref(it), C.byref(res)), "helmholtz")
        return u, (bool(ok), int(it.value), float(res.value))

    def pcg_laplace(self, x, b, max_iter, tol):
        """the reference's pcg on Poisson's operator for a given b"""
        x = _f(x).copy()
        it, res = C.c_int(), C.c_double()
        ok = _check(lib().ref_pcg_laplace(self._h, _p(x), _p(_f(b)), int(max_iter), float(tol), C.byref(it),
                                          C.byref(res)), "pcg")
        return x, (bool(ok), int(it.value), float(res.value))

    def minres_helmholtz(self, c, x, b, max_iter, tol):
        """the reference's minres on Helmholtz's operator for a given b"""
        x = _f(x).copy()
        it, res = C.c_int(), C.c_double()
        ok = _check(lib().ref_minres_helmholtz(self._h, _p(_f(c)), _p(x), _p(_f(b)), int(max_iter), float(tol),
                                               C.byref(it), C.byref(res)), "minres")
        return x, (bool(ok), int(it.value), float(res.value))

    def dirichlet_bc(self, helm, c, u, f, g, max_iter, tol):
        """Inhomogeneous Dirichlet data by lifting, composed of the
        reference's own gproj, galerkin operators, mask, unmask and
        PCG/MINRES: u_D = g at every copy of a boundary node (0 elsewhere),
        b = gproj(f) - A u_D, A u0 = b, u = unmask(u0) + u_D"""
        X = self.zeros()
        t, ptr, el, ii, jj = self.nodes()
        E = self.edges()
        g = _f(g)
        N = self.N
        k = np.arange(N)
        sides = {1: (np.zeros(N, int), k), 2: (k, np.full(N, N - 1)), 3: (np.full(N, N - 1), k),
                 4: (k, np.zeros(N, int))}  # reference side -> (j, i)
        for row in E:
            if row[6]:
                e, s = int(row[0]), int(row[2])
                j_, i_ = sides[s]
                X[e, j_, i_] = g[e, j_, i_]
        for n in range(self.n_nodes):
            if t[n]:
                for q in range(ptr[n], ptr[n + 1]):
                    X[el[q], jj[q], ii[q]] = g[el[q], jj[q], ii[q]]
        b = self.gproj(f) - (self.apply_helmholtz(c, X) if helm else self.apply_laplace(X))
        x0 = self.mask(u)
        x, r = self.minres_helmholtz(c, x0, b, max_iter, tol) if helm else self.pcg_laplace(x0, b, max_iter, tol)
        return self.unmask(x) + X, r

    def minres_res(self, V, alpha, b_re, b_im, x_re, x_im, max_iter, tol):
        xr, xi = _f(x_re).copy(), _f(x_im).copy()
        it, res = C.c_int(), C.c_double()
        ok = _check(lib().ref_minres_res(self._h, _p(_f(V)), float(alpha), _p(_f(b_re)), _p(_f(b_im)), _p(xr),
                                         _p(xi), int(max_iter), float(tol), C.byref(it), C.byref(res)),
                    "minres")
        return xr, xi, (bool(ok), int(it.value), float(res.value))

    def schrodinger(self, method: str, psi_re, psi_im, V, dt, max_iter, tol, n_steps, untimed=0,
                    budget_s=0.0):
        """Run the reference's driver for n_steps steps (fewer once the steps
        after the first ``untimed`` have taken ``budget_s`` seconds, when
        given).  Returns (re, im, success, steps_done, per-step wall seconds)."""
        pr, pi = _f(psi_re).copy(), _f(psi_im).copy()
        times = np.zeros(max(int(n_steps), 1))
        done = C.c_int()
        ok = _check(lib().ref_schrodinger(self._h, METHODS[method], _p(pr), _p(pi), _p(_f(V)), float(dt),
                                          int(max_iter), float(tol), int(n_steps), int(untimed), float(budget_s),
                                          _p(times), C.byref(done)), "schrodinger")
        return pr, pi, bool(ok), int(done.value), times[: int(done.value)]
