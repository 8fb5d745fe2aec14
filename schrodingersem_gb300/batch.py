"""Python view of a ``sem_batch``: many independent Schroedinger instances
(each its own mesh, degree, potential and state) advanced together by the
reference's BDF2 driver with the mixed-precision stage solve, one
persistent launch per time step replayed from a captured CUDA graph."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import SemBatchStats, SemMeshInfo, SemSolverOpts, check


def _torch():
    import torch
    return torch


def _ptr(a):
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"] and a.dtype == np.float64
        return a.ctypes.data
    torch = _torch()
    if not (isinstance(a, torch.Tensor) and a.is_cuda and a.is_contiguous() and a.dtype == torch.float64):
        raise TypeError("expected a host float64 array or a contiguous CUDA float64 tensor")
    return a.data_ptr()


class Batch:
    def __init__(self, meshes, corrected_metric: bool = False, stream=None):
        """meshes: list of (p, coords (n_nodes x 2), elements (n_el x 4))"""
        L = capi.load()
        self._L = L
        n = len(meshes)
        self._keep = []
        ps = (C.c_int * n)(*[int(m[0]) for m in meshes])
        nn = (C.c_int * n)()
        ne = (C.c_int * n)()
        cp = (C.c_void_p * n)()
        ep = (C.c_void_p * n)()
        for i, (p, co, el) in enumerate(meshes):
            co = np.ascontiguousarray(co, dtype=np.float64).reshape(-1, 2)
            el = np.ascontiguousarray(el, dtype=np.int32).reshape(-1, 4)
            self._keep += [co, el]
            nn[i], ne[i] = co.shape[0], el.shape[0]
            cp[i], ep[i] = co.ctypes.data, el.ctypes.data
        h = C.c_void_p()
        flags = capi.SEM_FLAG_METRIC_CORRECTED if corrected_metric else 0
        check(L.sem_batch_create(C.byref(h), n, ps, nn, C.cast(cp, C.POINTER(C.c_void_p)), ne,
                                 C.cast(ep, C.POINTER(C.c_void_p)), flags), "sem_batch_create")
        self._h = h
        self.n = n
        self.info = []
        for i in range(n):
            inf = SemMeshInfo()
            check(L.sem_batch_get_info(h, i, C.byref(inf)), "sem_batch_get_info")
            self.info.append(inf)
        torch = _torch()
        if stream is None and torch.cuda.is_available():
            stream = torch.cuda.current_stream()
        if stream is not None:
            check(L.sem_batch_set_stream(h, C.c_void_p(stream.cuda_stream)), "sem_batch_set_stream")

    def close(self):
        if getattr(self, "_h", None):
            self._L.sem_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, i):
        inf = self.info[i]
        return (inf.n_elements, inf.N, inf.N)

    def set_option(self, opt: int, value: float):
        check(self._L.sem_batch_set_option(self._h, int(opt), float(value)), "sem_batch_set_option")

    def stats(self) -> SemBatchStats:
        s = SemBatchStats()
        check(self._L.sem_batch_get_stats(self._h, C.byref(s)), "sem_batch_get_stats")
        return s

    def instance(self, i):
        steps, stopped, its = C.c_int(), C.c_int(), C.c_longlong()
        check(self._L.sem_batch_get_instance(self._h, int(i), C.byref(steps), C.byref(stopped), C.byref(its)),
              "sem_batch_get_instance")
        return int(steps.value), bool(stopped.value), int(its.value)

    def bdf2(self, psi_re, psi_im, V, T, dt, max_iter, tol):
        """schrodinger_bdf2 on every instance in place; returns per-instance success"""
        n = self.n
        arr = lambda xs: (C.c_void_p * n)(*[_ptr(x) for x in xs])  # noqa: E731
        pr, pi, pv = arr(psi_re), arr(psi_im), arr(V)
        ok = (C.c_int * n)()
        opts = SemSolverOpts(int(max_iter), float(tol), float(dt), 0)
        check(self._L.sem_batch_schrodinger_bdf2(self._h, C.cast(pr, C.POINTER(C.c_void_p)),
                                                 C.cast(pi, C.POINTER(C.c_void_p)),
                                                 C.cast(pv, C.POINTER(C.c_void_p)), float(T), C.byref(opts), ok),
              "sem_batch_schrodinger_bdf2")
        return [bool(v) for v in ok]
