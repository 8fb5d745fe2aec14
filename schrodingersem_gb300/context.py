"""Python view of one ``sem_ctx``: a mesh with its device data.

Device fields are torch CUDA tensors of dtype float64 (float32 for the
``*_f32`` calls) holding E*N*N values in the reference's element-local
column-major order; ``shape`` is (E, N, N) indexed [e, j, i].  Host fields
are numpy arrays with the same layout.  torch is used only to own device
memory and to name the stream; all arithmetic runs in the library's kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import SemMeshInfo, SemSolverOpts, SemSolverResults, SemStats, check


def _torch():
    import torch
    return torch


def _dptr(t, dtype=None):
    """device pointer of a contiguous CUDA tensor"""
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return C.c_void_p(t.data_ptr())


def _hptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"] and a.dtype == np.float64
    return C.c_void_p(a.ctypes.data)


def _ptr(a):
    """pointer of a host (numpy float64) or device (torch float64) field"""
    if isinstance(a, np.ndarray):
        return _hptr(a)
    return _dptr(a, _torch().float64)


class Context:
    def __init__(self, p: int, coords=None, elements=None, folder: str | None = None,
                 corrected_metric: bool = False, stream=None, neumann: bool = False):
        L = capi.load()
        self._L = L
        h = C.c_void_p()
        flags = (capi.SEM_FLAG_METRIC_CORRECTED if corrected_metric else 0) | \
            (capi.SEM_FLAG_NEUMANN if neumann else 0)
        self.neumann = bool(neumann)
        if folder is not None:
            check(L.sem_ctx_load(C.byref(h), int(p), folder.encode(), flags), "sem_ctx_load")
        else:
            co = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 2)
            el = np.ascontiguousarray(elements, dtype=np.int32).reshape(-1, 4)
            check(L.sem_ctx_create(C.byref(h), int(p), co.shape[0], co.ctypes.data_as(C.POINTER(C.c_double)),
                                   el.shape[0], el.ctypes.data_as(C.POINTER(C.c_int)), flags), "sem_ctx_create")
        self._h = h
        info = SemMeshInfo()
        check(L.sem_ctx_get_info(h, C.byref(info)), "sem_ctx_get_info")
        self.info = info
        self.p, self.N, self.E = info.p, info.N, info.n_elements
        self.n = info.n_local
        torch = _torch()
        if stream is None and torch.cuda.is_available():
            stream = torch.cuda.current_stream()
        if stream is not None:
            check(L.sem_ctx_set_stream(h, C.c_void_p(stream.cuda_stream)), "sem_ctx_set_stream")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sem_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- info
    @property
    def shape(self):
        return (self.E, self.N, self.N)

    def dof(self) -> int:
        return int(self.info.dof)

    def quadrature(self):
        x, w, D = np.zeros(self.N), np.zeros(self.N), np.zeros(self.N * self.N)
        check(self._L.sem_ctx_get_quadrature(self._h, _hptr(x), _hptr(w), _hptr(D)), "quadrature")
        return x, w, D.reshape(self.N, self.N).T.copy()

    def metrics(self):
        out = [np.zeros(self.shape) for _ in range(4)]
        check(self._L.sem_ctx_get_metrics(self._h, *[_hptr(a) for a in out]), "metrics")
        return out

    def node_coords(self):
        X, Y = np.zeros(self.shape), np.zeros(self.shape)
        check(self._L.sem_ctx_get_node_coords(self._h, _hptr(X), _hptr(Y)), "node_coords")
        return X, Y

    def set_option(self, opt: int, value: float):
        check(self._L.sem_ctx_set_option(self._h, int(opt), float(value)), "set_option")

    def stats(self) -> SemStats:
        s = SemStats()
        check(self._L.sem_ctx_get_stats(self._h, C.byref(s)), "stats")
        return s

    # ------------------------------------------------- learned stage guess
    def set_learner(self, learner):
        """network for SEM_GUESS_LEARNED (None: extrapolation only); the
        caller keeps the Learner alive while the context uses it"""
        self._learner = learner
        check(self._L.sem_ctx_set_learner(self._h, learner.handle if learner is not None else None),
              "sem_ctx_set_learner")

    def record(self, capacity_rows: int):
        """start recording training rows from the SDIRK stage solves"""
        check(self._L.sem_ctx_record(self._h, C.c_longlong(int(capacity_rows))), "sem_ctx_record")

    def dataset(self):
        """copies of the recorded rows: (X bf16 (rows, 4N^2), T float32 (rows, 2N^2))"""
        from .learned import device_view
        torch = _torch()
        X, T = C.c_void_p(), C.c_void_p()
        rows, di, do = C.c_longlong(0), C.c_int(0), C.c_int(0)
        check(self._L.sem_ctx_dataset(self._h, C.byref(X), C.byref(T), C.byref(rows), C.byref(di), C.byref(do)),
              "sem_ctx_dataset")
        torch.cuda.current_stream().synchronize()
        r = int(rows.value)
        Xv = device_view(X.value or 0, (r, di.value), torch.bfloat16).clone()
        Tv = device_view(T.value or 0, (r, do.value), torch.float32).clone()
        return Xv, Tv

    # ------------------------------------------------------- device helpers
    def zeros(self, dtype=None, planes: int = 1):
        torch = _torch()
        dtype = dtype or torch.float64
        shape = self.shape if planes == 1 else (planes,) + self.shape
        return torch.zeros(shape, dtype=dtype, device="cuda")

    def to_device(self, a: np.ndarray, dtype=None):
        torch = _torch()
        return torch.as_tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype or torch.float64)

    # ------------------------------------------------------ gather-scatter
    def unmask(self, a):
        check(self._L.sem_unmask(self._h, _dptr(a)), "sem_unmask")
        return a

    def global_sum(self, a):
        check(self._L.sem_global_sum(self._h, _dptr(a)), "sem_global_sum")
        return a

    def mask(self, a):
        check(self._L.sem_mask(self._h, _dptr(a)), "sem_mask")
        return a

    def dot(self, a, b) -> float:
        r = C.c_double()
        check(self._L.sem_dot(self._h, _dptr(a), _dptr(b), C.byref(r)), "sem_dot")
        return r.value

    def axpby(self, a, x, b, y, out):
        check(self._L.sem_vec_axpby(self._h, x.numel(), float(a), _dptr(x), float(b),
                                    _dptr(y) if y is not None else None, _dptr(out)), "sem_vec_axpby")
        return out

    # ------------------------------------------------------------ operators
    def gproj(self, u, out=None):
        out = self.zeros() if out is None else out
        check(self._L.sem_gproj(self._h, _dptr(u), _dptr(out)), "sem_gproj")
        return out

    def apply_laplace(self, u, out=None):
        out = self.zeros() if out is None else out
        check(self._L.sem_apply_laplace(self._h, _dptr(u), _dptr(out)), "sem_apply_laplace")
        return out

    def apply_helmholtz(self, c, u, out=None):
        out = self.zeros() if out is None else out
        check(self._L.sem_apply_helmholtz(self._h, _dptr(c), _dptr(u), _dptr(out)), "sem_apply_helmholtz")
        return out

    def schro_res(self, V, alpha, qr, qi, yr=None, yi=None):
        yr = self.zeros() if yr is None else yr
        yi = self.zeros() if yi is None else yi
        check(self._L.sem_apply_schro_res(self._h, _dptr(V), float(alpha), _dptr(qr), _dptr(qi),
                                          _dptr(yr), _dptr(yi)), "sem_apply_schro_res")
        return yr, yi

    def schro_f(self, V, qr, qi, yr=None, yi=None):
        yr = self.zeros() if yr is None else yr
        yi = self.zeros() if yi is None else yi
        check(self._L.sem_apply_schro_f(self._h, _dptr(V), _dptr(qr), _dptr(qi), _dptr(yr), _dptr(yi)),
              "sem_apply_schro_f")
        return yr, yi

    def schro_res_f32(self, V, alpha, qr, qi, yr=None, yi=None):
        torch = _torch()
        yr = self.zeros(torch.float32) if yr is None else yr
        yi = self.zeros(torch.float32) if yi is None else yi
        f = torch.float32
        check(self._L.sem_apply_schro_res_f32(self._h, _dptr(V, f), float(alpha), _dptr(qr, f), _dptr(qi, f),
                                              _dptr(yr, f), _dptr(yi, f)), "sem_apply_schro_res_f32")
        return yr, yi

    # ------------------------------------------------------------- solvers
    def minres_schro(self, V, alpha, xr, xi, br, bi, maxit, tol, x_is_zero=False):
        r = SemSolverResults()
        check(self._L.sem_minres_schro(self._h, _dptr(V), float(alpha), _dptr(xr), _dptr(xi), _dptr(br),
                                       _dptr(bi), int(maxit), float(tol), int(bool(x_is_zero)), C.byref(r)),
              "sem_minres_schro")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def minres_helmholtz(self, c, x, b, maxit, tol, x_is_zero=False):
        r = SemSolverResults()
        check(self._L.sem_minres_helmholtz(self._h, _dptr(c), _dptr(x), _dptr(b), int(maxit), float(tol),
                                           int(bool(x_is_zero)), C.byref(r)), "sem_minres_helmholtz")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def pcg_laplace(self, x, b, max_iter, tol, x_is_zero=False):
        r = SemSolverResults()
        check(self._L.sem_pcg_laplace(self._h, _dptr(x), _dptr(b), int(max_iter), float(tol),
                                      int(bool(x_is_zero)), C.byref(r)), "sem_pcg_laplace")
        return bool(r.success), int(r.n_iter), float(r.residual)

    # ------------------------------------------------------------- drivers
    def poisson(self, u, f, max_iter, tol):
        r = SemSolverResults()
        check(self._L.sem_poisson(self._h, _ptr(u), _ptr(f), int(max_iter), float(tol), C.byref(r)),
              "sem_poisson")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def helmholtz(self, u, c, f, max_iter, tol):
        r = SemSolverResults()
        check(self._L.sem_helmholtz(self._h, _ptr(u), _ptr(c), _ptr(f), int(max_iter), float(tol), C.byref(r)),
              "sem_helmholtz")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def poisson_bc(self, u, f, g, max_iter, tol):
        """sem_poisson_bc: u (host or device) in/out, continuous on return;
        g element-local (Dirichlet context) or (E, 4, N) normal derivatives
        per side node (Neumann context)"""
        r = SemSolverResults()
        check(self._L.sem_poisson_bc(self._h, _ptr(u), _ptr(f), _ptr(g), int(max_iter), float(tol), C.byref(r)),
              "sem_poisson_bc")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def helmholtz_bc(self, u, c, f, g, max_iter, tol):
        r = SemSolverResults()
        check(self._L.sem_helmholtz_bc(self._h, _ptr(u), _ptr(c), _ptr(f), _ptr(g), int(max_iter), float(tol),
                                       C.byref(r)), "sem_helmholtz_bc")
        return bool(r.success), int(r.n_iter), float(r.residual)

    def schrodinger_adaptive(self, psi_re, psi_im, V, T, dt0, max_iter, tol, err_tol, capacity=100000,
                             n_steps=None):
        """adaptive SDIRK4 5-stage in place (stops after n_steps accepted steps
        when given); returns (success, accepted dts, rejected count)"""
        opts = SemSolverOpts(int(max_iter), float(tol), float(dt0), 0)
        dts = np.zeros(int(capacity))
        na, nr, ok = C.c_int(0), C.c_int(0), C.c_int(0)
        cb = (capi.STEP_CALLBACK(lambda user, step, a, b: 1 if step >= n_steps else 0) if n_steps
              else capi.STEP_CALLBACK())
        check(self._L.sem_schrodinger_dirk4s5_adaptive(self._h, _ptr(psi_re), _ptr(psi_im), _ptr(V), float(T),
                                                       C.byref(opts), float(err_tol), _hptr(dts), int(capacity),
                                                       C.byref(na), C.byref(nr), cb, None, C.byref(ok)),
              "sem_schrodinger_dirk4s5_adaptive")
        return bool(ok.value), dts[:min(na.value, capacity)].copy(), int(nr.value)

    def schrodinger(self, method: str, psi_re, psi_im, V, T, dt, max_iter, tol, n_steps=None, record=None):
        """Run a driver in place on psi_re/psi_im (host numpy or device
        torch).  Stops after n_steps through the callback when given;
        ``record`` receives (step, stage_iters) per step."""
        fn = {"bdf2": self._L.sem_schrodinger_bdf2, "dirk4s5": self._L.sem_schrodinger_dirk4s5,
              "dirk4s3": self._L.sem_schrodinger_dirk4s3}[method]
        opts = SemSolverOpts(int(max_iter), float(tol), float(dt), 0)
        ok = C.c_int(0)

        def _cb(user, step, a, b):
            if record is not None:
                st = self.stats()
                record.append((int(step), [int(st.last_stage_iters[k]) for k in range(st.last_step_stages)]))
            return 1 if (n_steps is not None and step >= n_steps) else 0

        need_cb = (n_steps is not None) or (record is not None)
        cb = capi.STEP_CALLBACK(_cb) if need_cb else capi.STEP_CALLBACK()
        check(fn(self._h, _ptr(psi_re), _ptr(psi_im), _ptr(V), float(T), C.byref(opts), cb, None, C.byref(ok)),
              "sem_schrodinger_" + method)
        return bool(ok.value)
