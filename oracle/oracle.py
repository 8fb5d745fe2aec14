"""ctypes loader for the CPU oracle (``oracle/sem_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker the CUDA library is
compared against; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import this module.  The product package
never imports it.

Fields are numpy float64 arrays of shape (E, N, N) indexed ``a[e, j, i]``
(so that ``a.reshape(-1)`` is the reference's column-major element-local
layout: value (i, j) of element e at ``e*N*N + j*N + i``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsem_oracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _OrMesh(C.Structure):
    _fields_ = [
        ("p", C.c_int), ("N", C.c_int), ("n_nodes", C.c_int), ("n_el", C.c_int), ("n_edges", C.c_int),
        ("x", _dp), ("w", _dp), ("D", _dp),
        ("xs", _dp), ("ys", _dp), ("corner_ids", _ip),
        ("edge_type", _ip), ("edge_el", _ip), ("edge_side", _ip), ("edge_start", _ip), ("edge_delta", _ip),
        ("node_type", _ip), ("node_x", _dp), ("node_y", _dp),
        ("node_ptr", _ip), ("node_el", _ip), ("node_i", _ip), ("node_j", _ip),
        ("J", _dp), ("A", _dp), ("B", _dp), ("C", _dp),
    ]


class OrResults(C.Structure):
    _fields_ = [("success", C.c_int), ("n_iter", C.c_int), ("residual", C.c_double)]


class OrOpts(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("tol", C.c_double), ("dt", C.c_double), ("verbose", C.c_int)]


_CB = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, _dp, _dp, _ip, C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.or_gauss_lobatto.argtypes = [C.c_int, _dp, _dp]
        L.or_derivative_matrix.argtypes = [C.c_int, _dp, _dp]
        L.or_legendre_p.argtypes = [C.c_int, C.c_double]
        L.or_legendre_p.restype = C.c_double
        L.or_mesh_create.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip]
        L.or_mesh_create.restype = C.POINTER(_OrMesh)
        L.or_mesh_load.argtypes = [C.c_int, C.c_char_p]
        L.or_mesh_load.restype = C.POINTER(_OrMesh)
        L.or_mesh_compute_metrics.argtypes = [C.POINTER(_OrMesh), C.c_int]
        L.or_mesh_set_neumann.argtypes = [C.POINTER(_OrMesh)]
        L.or_mesh_free.argtypes = [C.POINTER(_OrMesh)]
        L.or_mesh_dof.argtypes = [C.POINTER(_OrMesh)]
        L.or_mesh_node_coords.argtypes = [C.POINTER(_OrMesh), _dp, _dp]
        for fn in ("or_unmask", "or_global_sum", "or_mask"):
            getattr(L, fn).argtypes = [C.POINTER(_OrMesh), _dp]
        L.or_dot.argtypes = [C.POINTER(_OrMesh), _dp, _dp]
        L.or_dot.restype = C.c_double
        L.or_glaplace.argtypes = [C.POINTER(_OrMesh), C.c_int, _dp, _dp]
        L.or_gproj.argtypes = [C.POINTER(_OrMesh), _dp, _dp]
        L.or_apply_laplace.argtypes = [C.POINTER(_OrMesh), _dp, _dp]
        L.or_apply_helmholtz.argtypes = [C.POINTER(_OrMesh), _dp, _dp, _dp]
        L.or_schro_res.argtypes = [C.POINTER(_OrMesh), _dp, C.c_double, _dp, _dp, _dp, _dp]
        L.or_schro_f.argtypes = [C.POINTER(_OrMesh), _dp, _dp, _dp, _dp, _dp]
        L.or_poisson.argtypes = [C.POINTER(_OrMesh), _dp, _dp, C.c_int, C.c_double]
        L.or_poisson.restype = OrResults
        L.or_helmholtz.argtypes = [C.POINTER(_OrMesh), _dp, _dp, _dp, C.c_int, C.c_double]
        L.or_helmholtz.restype = OrResults
        for fn in ("or_schrodinger_bdf2", "or_schrodinger_dirk4s5", "or_schrodinger_dirk4s3"):
            getattr(L, fn).argtypes = [C.POINTER(_OrMesh), _dp, _dp, _dp, C.c_double, C.POINTER(OrOpts),
                                       _CB, C.c_void_p]
            getattr(L, fn).restype = C.c_int
        L.or_minres.argtypes = [_dp, C.c_void_p, C.c_void_p, _dp, C.c_void_p, C.c_void_p, C.c_long,
                                C.c_int, C.c_double]
        L.or_minres.restype = OrResults
        L.or_pcg.argtypes = L.or_minres.argtypes
        L.or_pcg.restype = OrResults
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        _lib = L
    return _lib


_LINOP = C.CFUNCTYPE(None, C.c_void_p, _dp, _dp)
_DOTFN = C.CFUNCTYPE(C.c_double, C.c_void_p, _dp, _dp)


def krylov(method: str, apply, b: np.ndarray, x0: np.ndarray, maxit: int, tol: float, dot=None):
    """The oracle's generic minres / pcg (include/minres.hpp, include/pcg.hpp)
    on a Python operator ``apply(v) -> A v`` over flat float64 vectors."""
    n = b.size

    def _op(ctx, a, out):
        v = np.ctypeslib.as_array(a, (n,)).copy()
        np.ctypeslib.as_array(out, (n,))[:] = apply(v)

    def _dot(ctx, a, c):
        av = np.ctypeslib.as_array(a, (n,))
        cv = np.ctypeslib.as_array(c, (n,))
        return float(dot(av, cv)) if dot else float(np.dot(av, cv))

    op_cb, dot_cb = _LINOP(_op), _DOTFN(_dot)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    bb = np.ascontiguousarray(b, dtype=np.float64)
    fn = lib().or_minres if method == "minres" else lib().or_pcg
    r = fn(_p(x), C.cast(op_cb, C.c_void_p), None, _p(bb), C.cast(dot_cb, C.c_void_p), None, n,
           int(maxit), float(tol))
    return x, (bool(r.success), int(r.n_iter), float(r.residual))


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return int(lib().or_get_threads())


def gauss_lobatto(p: int):
    x = np.zeros(p + 1)
    w = np.zeros(p + 1)
    if lib().or_gauss_lobatto(int(p), _p(x), _p(w)) != 0:
        raise ValueError("gauss_lobatto: p must be >= 1")
    return x, w


def derivative_matrix(x: np.ndarray) -> np.ndarray:
    """D with D[i, j] = d l_j / dx (x_i) (row i, column j)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = x.size
    Dc = np.zeros(n * n)
    lib().or_derivative_matrix(n, _p(x), _p(Dc))
    return Dc.reshape(n, n).T.copy()  # column-major -> [i, j]


def legendre_p(n: int, x: float) -> float:
    return float(lib().or_legendre_p(int(n), float(x)))


class Mesh:
    """The oracle's mesh: topology (load_mesh.hpp) + metrics (Quad.hpp)."""

    def __init__(self, p: int, coords=None, elements=None, folder: str | None = None, ref_compat: bool = True,
                 neumann: bool = False):
        L = lib()
        if folder is not None:
            ptr = L.or_mesh_load(int(p), folder.encode())
        else:
            co = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 2)
            el = np.ascontiguousarray(elements, dtype=np.int32).reshape(-1, 4)
            self._co, self._el = co, el
            ptr = L.or_mesh_create(int(p), co.shape[0], _p(co), el.shape[0], el.ctypes.data_as(_ip))
        if not ptr:
            raise ValueError("oracle: could not build mesh")
        self._ptr = ptr
        L.or_mesh_compute_metrics(ptr, 1 if ref_compat else 0)
        self.neumann = bool(neumann)
        if neumann:
            L.or_mesh_set_neumann(ptr)
        m = ptr.contents
        self.p, self.N, self.n_nodes, self.n_el, self.n_edges = m.p, m.N, m.n_nodes, m.n_el, m.n_edges
        N, E = self.N, self.n_el
        self.x = np.ctypeslib.as_array(m.x, (N,)).copy()
        self.w = np.ctypeslib.as_array(m.w, (N,)).copy()
        self.D = np.ctypeslib.as_array(m.D, (N * N,)).reshape(N, N).T.copy()
        self.edge_type = np.ctypeslib.as_array(m.edge_type, (self.n_edges,)).copy()
        self.edge_el = np.ctypeslib.as_array(m.edge_el, (self.n_edges * 2,)).reshape(-1, 2).copy()
        self.edge_side = np.ctypeslib.as_array(m.edge_side, (self.n_edges * 2,)).reshape(-1, 2).copy()
        self.node_type = np.ctypeslib.as_array(m.node_type, (self.n_nodes,)).copy()
        self.node_ptr = np.ctypeslib.as_array(m.node_ptr, (self.n_nodes + 1,)).copy()
        self.node_el = np.ctypeslib.as_array(m.node_el, (4 * E,)).copy()
        self.corner_ids = np.ctypeslib.as_array(m.corner_ids, (4 * E,)).reshape(E, 4).copy()
        self.xs = np.ctypeslib.as_array(m.xs, (4 * E,)).reshape(E, 4).copy()
        self.ys = np.ctypeslib.as_array(m.ys, (4 * E,)).reshape(E, 4).copy()
        self.node_i = np.ctypeslib.as_array(m.node_i, (4 * E,)).copy()
        self.node_j = np.ctypeslib.as_array(m.node_j, (4 * E,)).copy()
        sh = (E, N, N)
        self.J = np.ctypeslib.as_array(m.J, (E * N * N,)).reshape(sh).copy()
        self.A = np.ctypeslib.as_array(m.A, (E * N * N,)).reshape(sh).copy()
        self.B = np.ctypeslib.as_array(m.B, (E * N * N,)).reshape(sh).copy()
        self.C = np.ctypeslib.as_array(m.C, (E * N * N,)).reshape(sh).copy()

    def __del__(self):
        try:
            if getattr(self, "_ptr", None):
                lib().or_mesh_free(self._ptr)
                self._ptr = None
        except Exception:
            pass

    @property
    def shape(self):
        return (self.n_el, self.N, self.N)

    def zeros(self):
        return np.zeros(self.shape)

    def dof(self) -> int:
        return int(lib().or_mesh_dof(self._ptr))

    def node_coords(self):
        X, Y = self.zeros(), self.zeros()
        lib().or_mesh_node_coords(self._ptr, _p(X), _p(Y))
        return X, Y

    # ---- L3 ----
    def unmask(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        lib().or_unmask(self._ptr, _p(a))
        return a

    def global_sum(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        lib().or_global_sum(self._ptr, _p(a))
        return a

    def mask(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).copy()
        lib().or_mask(self._ptr, _p(a))
        return a

    def dot(self, a, b) -> float:
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        return float(lib().or_dot(self._ptr, _p(a), _p(b)))

    # ---- L1/L5 ----
    def glaplace(self, e: int, u_e):
        u = np.ascontiguousarray(u_e, dtype=np.float64)
        out = np.zeros_like(u)
        lib().or_glaplace(self._ptr, int(e), _p(u), _p(out))
        return out

    def gproj(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = self.zeros()
        lib().or_gproj(self._ptr, _p(u), _p(out))
        return out

    def apply_laplace(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = self.zeros()
        lib().or_apply_laplace(self._ptr, _p(u), _p(out))
        return out

    def apply_helmholtz(self, c, u):
        c = np.ascontiguousarray(c, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = self.zeros()
        lib().or_apply_helmholtz(self._ptr, _p(c), _p(u), _p(out))
        return out

    def schro_res(self, V, alpha, q_re, q_im):
        V, q_re, q_im = (np.ascontiguousarray(t, dtype=np.float64) for t in (V, q_re, q_im))
        y_re, y_im = self.zeros(), self.zeros()
        lib().or_schro_res(self._ptr, _p(V), float(alpha), _p(q_re), _p(q_im), _p(y_re), _p(y_im))
        return y_re, y_im

    def schro_f(self, V, q_re, q_im):
        V, q_re, q_im = (np.ascontiguousarray(t, dtype=np.float64) for t in (V, q_re, q_im))
        y_re, y_im = self.zeros(), self.zeros()
        lib().or_schro_f(self._ptr, _p(V), _p(q_re), _p(q_im), _p(y_re), _p(y_im))
        return y_re, y_im

    # ---- L7 ----
    def poisson(self, u, f, max_iter, tol):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        f = np.ascontiguousarray(f, dtype=np.float64)
        r = lib().or_poisson(self._ptr, _p(u), _p(f), int(max_iter), float(tol))
        return u, (bool(r.success), int(r.n_iter), float(r.residual))

    def helmholtz(self, u, c, f, max_iter, tol):
        u = np.ascontiguousarray(u, dtype=np.float64).copy()
        c = np.ascontiguousarray(c, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        r = lib().or_helmholtz(self._ptr, _p(u), _p(c), _p(f), int(max_iter), float(tol))
        return u, (bool(r.success), int(r.n_iter), float(r.residual))

    def schrodinger(self, method: str, psi_re, psi_im, V, T, dt, max_iter, tol, n_steps=None,
                    record=None):
        """Run one of the reference's drivers; stops after n_steps steps
        through the callback hook when given.  ``record`` (a list) receives
        (step, stage_iters) per step."""
        fn = {"bdf2": lib().or_schrodinger_bdf2, "dirk4s5": lib().or_schrodinger_dirk4s5,
              "dirk4s3": lib().or_schrodinger_dirk4s3}[method]
        pr = np.ascontiguousarray(psi_re, dtype=np.float64).copy()
        pi = np.ascontiguousarray(psi_im, dtype=np.float64).copy()
        V = np.ascontiguousarray(V, dtype=np.float64)
        opts = OrOpts(int(max_iter), float(tol), float(dt), 0)

        def _cb(user, step, a, b, iters, n):
            if record is not None:
                record.append((int(step), [int(iters[k]) for k in range(n)]))
            return 1 if (n_steps is not None and step >= n_steps) else 0

        cb = _CB(_cb)
        ok = fn(self._ptr, _p(pr), _p(pi), _p(V), float(T), C.byref(opts), cb, None)
        return pr, pi, bool(ok)

    # ---- boundary data (no counterpart in the reference) ----
    def _side_index(self, s0: int):
        """(j, i) index arrays of the N nodes of library side s0 (0: j = 0,
        1: i = N-1, 2: j = N-1, 3: i = 0), k along the element's own i (sides
        0, 2) or j (sides 1, 3)"""
        N = self.N
        k = np.arange(N)
        return {0: (np.zeros(N, int), k), 1: (k, np.full(N, N - 1)), 2: (np.full(N, N - 1), k),
                3: (k, np.zeros(N, int))}[s0]

    def bc_field(self, g):
        """Dirichlet mesh: the lifting u_D (g at every copy of a boundary node,
        0 elsewhere), g element-local.  Neumann mesh: the boundary integral
        w_k (L/2) g[e, s, k] at node k of every boundary side s of length L,
        g of shape (E, 4, N) (outward normal derivative per side node)."""
        F = self.zeros()
        g = np.asarray(g, dtype=np.float64)
        ca, cb = (0, 1, 3, 0), (1, 2, 2, 3)
        for ed in range(self.n_edges):
            if self.edge_type[ed] != 1:
                continue
            e, s0 = int(self.edge_el[ed, 0]), int(self.edge_side[ed, 0]) - 1
            jj, ii = self._side_index(s0)
            if self.neumann:
                L = np.hypot(self.xs[e, cb[s0]] - self.xs[e, ca[s0]], self.ys[e, cb[s0]] - self.ys[e, ca[s0]])
                F[e, jj, ii] += self.w * (0.5 * L) * g[e, s0, :]
            else:
                F[e, jj, ii] = g[e, jj, ii]
        if not self.neumann:
            for c in range(self.n_nodes):
                if self.node_type[c] != 1:
                    continue
                for q in range(self.node_ptr[c], self.node_ptr[c + 1]):
                    e, i, j = self.node_el[q], self.node_i[q], self.node_j[q]
                    F[e, j, i] = g[e, j, i]
        return F

    def _bc(self, helm, c, u, f, g, max_iter, tol):
        sh = self.shape
        F = self.bc_field(g)
        b = self.gproj(f)

        def op(v):
            return self.apply_helmholtz(c, v) if helm else self.apply_laplace(v)
        if self.neumann:
            b = b + self.mask(self.global_sum(F))
        else:
            b = b - op(F)
        x0 = self.mask(u)
        x, r = krylov("minres" if helm else "pcg", lambda v: op(v.reshape(sh)).ravel(), b.ravel(), x0.ravel(),
                      max_iter, tol, dot=lambda a, d: self.dot(a.reshape(sh), d.reshape(sh)))
        x = self.unmask(x.reshape(sh))
        if not self.neumann:
            x = x + F
        return x, r

    def poisson_bc(self, u, f, g, max_iter, tol):
        """Poisson with boundary data g (see bc_field), the composition of
        sem_poisson_bc: Dirichlet by lifting, Neumann by the boundary
        integral; returns the continuous solution and (success, n_iter,
        residual)"""
        return self._bc(False, None, u, f, g, max_iter, tol)

    def helmholtz_bc(self, u, c, f, g, max_iter, tol):
        return self._bc(True, c, u, f, g, max_iter, tol)
