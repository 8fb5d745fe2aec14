"""Learned initial guess for the SDIRK stage solves (no counterpart in the
reference, whose stage solves start from zero: schrodinger.hpp:222,379).

``Learner`` wraps the library's per-element MLP (``sem_learner_*``): BF16
tensor-core GEMMs with FP32 accumulation, FP32 master weights and Adam, all
on the GPU in the library's own kernels.  torch tensors only carry device
memory in and out.

Rows are elements.  Input row (4 N^2 BF16 values): the residual of the
extrapolated stage guess scaled by the element's RMS residual rho (real and
imaginary planes), alpha V and the lumped mass over alpha.  Output row
(2 N^2): the predicted correction (z - z_guess) mbar / rho, mbar the
element's mean lumped mass.  ``Context.record``
collects such rows from solved stages; ``Learner.fit`` trains on them;
``Context.set_learner`` makes the drivers use the network, with the
extrapolation kept whenever the network's guess has the larger FP64
residual.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check


def _torch():
    import torch
    return torch


def _dev(t, dtype):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous() or t.dtype != dtype:
        raise TypeError(f"expected a contiguous CUDA tensor of {dtype}")
    return C.c_void_p(t.data_ptr())


class _DevView:
    """__cuda_array_interface__ over device memory the library owns"""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(int(s) for s in shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3, "strides": None}


def device_view(ptr: int, shape, dtype):
    """torch tensor aliasing library-owned device memory (no copy)"""
    torch = _torch()
    if int(np.prod(shape)) == 0 or not ptr:
        return torch.empty(shape, dtype=dtype, device="cuda")
    if dtype == torch.bfloat16:
        return torch.as_tensor(_DevView(ptr, shape, "<i2"), device="cuda").view(torch.bfloat16)
    ts = {torch.float32: "<f4", torch.float64: "<f8"}[dtype]
    return torch.as_tensor(_DevView(ptr, shape, ts), device="cuda")


class Learner:
    def __init__(self, d_in: int, hidden: int, d_out: int, seed: int = 1, stream=None):
        L = capi.load()
        self._L = L
        h = C.c_void_p()
        check(L.sem_learner_create(C.byref(h), int(d_in), int(hidden), int(d_out), C.c_ulonglong(int(seed))),
              "sem_learner_create")
        self._h = h
        self.d_in, self.hidden, self.d_out = int(d_in), int(hidden), int(d_out)
        torch = _torch()
        if stream is None and torch.cuda.is_available():
            stream = torch.cuda.current_stream()
        if stream is not None:
            check(L.sem_learner_set_stream(h, C.c_void_p(stream.cuda_stream)), "sem_learner_set_stream")

    @classmethod
    def for_mesh(cls, N: int, hidden: int = 256, seed: int = 1, stream=None):
        return cls(4 * N * N, hidden, 2 * N * N, seed, stream)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._L.sem_learner_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layer_shape(self, l: int):
        dims = [self.d_in, self.hidden, self.hidden, self.d_out]
        return dims[l], dims[l + 1]

    def params(self, l: int):
        i, o = self.layer_shape(l)
        W, b = np.zeros((i, o), np.float32), np.zeros(o, np.float32)
        check(self._L.sem_learner_get_params(self._h, int(l), C.c_void_p(W.ctypes.data), C.c_void_p(b.ctypes.data)),
              "sem_learner_get_params")
        return W, b

    def set_params(self, l: int, W, b):
        i, o = self.layer_shape(l)
        W = np.ascontiguousarray(W, np.float32).reshape(i, o)
        b = np.ascontiguousarray(b, np.float32).reshape(o)
        check(self._L.sem_learner_set_params(self._h, int(l), C.c_void_p(W.ctypes.data), C.c_void_p(b.ctypes.data)),
              "sem_learner_set_params")

    def grads(self, l: int):
        i, o = self.layer_shape(l)
        gW, gb = np.zeros((i, o), np.float32), np.zeros(o, np.float32)
        check(self._L.sem_learner_get_grads(self._h, int(l), C.c_void_p(gW.ctypes.data),
                                            C.c_void_p(gb.ctypes.data)), "sem_learner_get_grads")
        return gW, gb

    def forward(self, x):
        """x: CUDA bf16 (rows, d_in) -> CUDA float32 (rows, d_out)"""
        torch = _torch()
        out = torch.empty((x.shape[0], self.d_out), dtype=torch.float32, device="cuda")
        check(self._L.sem_learner_forward(self._h, int(x.shape[0]), _dev(x, torch.bfloat16),
                                          _dev(out, torch.float32)), "sem_learner_forward")
        return out

    def train_step(self, x, target, lr: float = 0.0) -> float:
        """mean-squared-error loss of one batch; gradients kept; lr > 0 takes an Adam step"""
        torch = _torch()
        loss = C.c_double(0.0)
        check(self._L.sem_learner_train_step(self._h, int(x.shape[0]), _dev(x, torch.bfloat16),
                                             _dev(target, torch.float32), C.c_float(lr), C.byref(loss)),
              "sem_learner_train_step")
        return float(loss.value)

    def fit(self, X, T, epochs: int = 20, batch: int = 256, lr: float = 1e-3, seed: int = 7) -> float:
        torch = _torch()
        loss = C.c_double(0.0)
        check(self._L.sem_learner_fit(self._h, _dev(X, torch.bfloat16), _dev(T, torch.float32),
                                      C.c_longlong(int(X.shape[0])), int(epochs), int(batch), C.c_float(lr),
                                      C.c_ulonglong(int(seed)), C.byref(loss)), "sem_learner_fit")
        return float(loss.value)


def gemm_bf16(A, B):
    """C = A @ B on the library's BF16 tensor-core GEMM (FP32 accumulate)"""
    torch = _torch()
    M, K = A.shape
    K2, N = B.shape
    if K != K2:
        raise ValueError("inner dimensions differ")
    Cm = torch.empty((M, N), dtype=torch.float32, device="cuda")
    check(capi.load().sem_gemm_bf16(int(M), int(N), int(K), _dev(A, torch.bfloat16), _dev(B, torch.bfloat16),
                                    _dev(Cm, torch.float32), C.c_void_p(torch.cuda.current_stream().cuda_stream)),
          "sem_gemm_bf16")
    return Cm
