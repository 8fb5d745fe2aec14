"""ctypes binding of the C ABI in include/sem_gb300.h.

This module only loads ``_lib/libsemgb300.so`` (built in-tree by
``schrodingersem_gb300.build``) and declares its entry points.  It has no
fallback: if the library is missing, importing it raises.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_vp = C.c_void_p


class SemSolverResults(C.Structure):
    _fields_ = [("success", C.c_int), ("n_iter", C.c_int), ("residual", C.c_double)]


class SemSolverOpts(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("tol", C.c_double), ("dt", C.c_double), ("verbose", C.c_int)]


class SemMeshInfo(C.Structure):
    _fields_ = [("p", C.c_int), ("N", C.c_int), ("n_elements", C.c_int), ("n_nodes", C.c_int),
                ("n_edges", C.c_int), ("n_interior_edges", C.c_int), ("n_boundary_edges", C.c_int),
                ("n_boundary_nodes", C.c_int), ("n_local", C.c_longlong), ("dof", C.c_longlong)]


class SemStats(C.Structure):
    _fields_ = [("krylov_iterations", C.c_longlong), ("fp64_applies", C.c_longlong),
                ("fp32_applies", C.c_longlong), ("last_step_stages", C.c_int),
                ("last_stage_iters", C.c_int * 8), ("last_stage_sweeps", C.c_int * 8),
                ("last_error_estimate", C.c_double), ("steps_taken", C.c_int),
                ("kernel_launches", C.c_longlong), ("solver_launches", C.c_longlong),
                ("solver_kernel_ms", C.c_double), ("solver_iterations_fp64", C.c_longlong),
                ("solver_iterations_fp32", C.c_longlong), ("learned_guesses", C.c_longlong),
                ("learned_accepted", C.c_longlong), ("last_guess_residual_ratio", C.c_double),
                ("last_guess_theta", C.c_double), ("learned_ratio_sum", C.c_double),
                ("resident_launches", C.c_longlong), ("projected_guesses", C.c_longlong),
                ("last_projection_ratio", C.c_double), ("projection_ratio_sum", C.c_double)]


class SemBatchStats(C.Structure):
    _fields_ = [("steps", C.c_longlong), ("instance_steps", C.c_longlong), ("krylov_iterations", C.c_longlong),
                ("graph_launches", C.c_longlong), ("graphs_built", C.c_longlong), ("kernel_ms", C.c_double),
                ("kmax_of_p", C.c_int * 17)]


STEP_CALLBACK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, _dp, _dp)

# name -> (restype, argtypes); every function declared in include/sem_gb300.h
SIGNATURES = {
    "sem_version": (C.c_int, []),
    "sem_status_string": (C.c_char_p, [C.c_int]),
    "sem_last_error": (C.c_char_p, []),
    "sem_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int, _dp, C.c_int, C.POINTER(C.c_int), C.c_uint]),
    "sem_ctx_load": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_char_p, C.c_uint]),
    "sem_ctx_destroy": (C.c_int, [_vp]),
    "sem_ctx_get_info": (C.c_int, [_vp, C.POINTER(SemMeshInfo)]),
    "sem_ctx_set_stream": (C.c_int, [_vp, _vp]),
    "sem_ctx_set_option": (C.c_int, [_vp, C.c_int, C.c_double]),
    "sem_ctx_get_stats": (C.c_int, [_vp, C.POINTER(SemStats)]),
    "sem_ctx_get_quadrature": (C.c_int, [_vp, _vp, _vp, _vp]),
    "sem_ctx_get_metrics": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "sem_ctx_get_node_coords": (C.c_int, [_vp, _vp, _vp]),
    "sem_unmask": (C.c_int, [_vp, _vp]),
    "sem_global_sum": (C.c_int, [_vp, _vp]),
    "sem_mask": (C.c_int, [_vp, _vp]),
    "sem_dot": (C.c_int, [_vp, _vp, _vp, _dp]),
    "sem_vec_axpby": (C.c_int, [_vp, C.c_longlong, C.c_double, _vp, C.c_double, _vp, _vp]),
    "sem_gproj": (C.c_int, [_vp, _vp, _vp]),
    "sem_apply_laplace": (C.c_int, [_vp, _vp, _vp]),
    "sem_apply_helmholtz": (C.c_int, [_vp, _vp, _vp, _vp]),
    "sem_apply_schro_res": (C.c_int, [_vp, _vp, C.c_double, _vp, _vp, _vp, _vp]),
    "sem_apply_schro_f": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "sem_apply_schro_res_f32": (C.c_int, [_vp, _vp, C.c_float, _vp, _vp, _vp, _vp]),
    "sem_apply_schro_res_noalloc": (C.c_int, [_vp, _vp, C.c_double, _vp, _vp, _vp, _vp]),
    "sem_minres_schro": (C.c_int, [_vp, _vp, C.c_double, _vp, _vp, _vp, _vp, C.c_int, C.c_double, C.c_int,
                                   C.POINTER(SemSolverResults)]),
    "sem_minres_helmholtz": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.c_int,
                                       C.POINTER(SemSolverResults)]),
    "sem_pcg_laplace": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_double, C.c_int, C.POINTER(SemSolverResults)]),
    "sem_poisson": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SemSolverResults)]),
    "sem_helmholtz": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SemSolverResults)]),
    "sem_poisson_bc": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SemSolverResults)]),
    "sem_helmholtz_bc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_double, C.POINTER(SemSolverResults)]),
    "sem_schrodinger_bdf2": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.POINTER(SemSolverOpts),
                                       STEP_CALLBACK, _vp, C.POINTER(C.c_int)]),
    "sem_schrodinger_dirk4s5": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.POINTER(SemSolverOpts),
                                          STEP_CALLBACK, _vp, C.POINTER(C.c_int)]),
    "sem_schrodinger_dirk4s3": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.POINTER(SemSolverOpts),
                                          STEP_CALLBACK, _vp, C.POINTER(C.c_int)]),
    "sem_schrodinger_dirk4s5_adaptive": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.POINTER(SemSolverOpts),
                                                   C.c_double, _vp, C.c_int, C.POINTER(C.c_int),
                                                   C.POINTER(C.c_int), STEP_CALLBACK, _vp, C.POINTER(C.c_int)]),
    "sem_learner_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int, C.c_int, C.c_ulonglong]),
    "sem_learner_destroy": (C.c_int, [_vp]),
    "sem_learner_shape": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sem_learner_set_stream": (C.c_int, [_vp, _vp]),
    "sem_learner_get_params": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "sem_learner_set_params": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "sem_learner_forward": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "sem_learner_train_step": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_float, _dp]),
    "sem_learner_get_grads": (C.c_int, [_vp, C.c_int, _vp, _vp]),
    "sem_learner_fit": (C.c_int, [_vp, _vp, _vp, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_ulonglong, _dp]),
    "sem_gemm_bf16": (C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
    "sem_gemm_set_path": (C.c_int, [C.c_int]),
    "sem_gemm_check_error": (C.c_int, [C.POINTER(C.c_int)]),
    "sem_ctx_set_learner": (C.c_int, [_vp, _vp]),
    "sem_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(_vp), C.POINTER(C.c_int), C.POINTER(_vp), C.c_uint]),
    "sem_batch_destroy": (C.c_int, [_vp]),
    "sem_batch_set_stream": (C.c_int, [_vp, _vp]),
    "sem_batch_set_option": (C.c_int, [_vp, C.c_int, C.c_double]),
    "sem_batch_get_info": (C.c_int, [_vp, C.c_int, C.POINTER(SemMeshInfo)]),
    "sem_batch_get_stats": (C.c_int, [_vp, C.POINTER(SemBatchStats)]),
    "sem_batch_get_instance": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_longlong)]),
    "sem_batch_schrodinger_bdf2": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), C.c_double,
                                             C.POINTER(SemSolverOpts), C.POINTER(C.c_int)]),
    "sem_ctx_record": (C.c_int, [_vp, C.c_longlong]),
    "sem_ctx_dataset": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int)]),
}

SEM_FLAG_METRIC_CORRECTED = 0x1
SEM_FLAG_NEUMANN = 0x2
OPT_SOLVE_PRECISION, OPT_INNER_TOL, OPT_STAGE_GUESS, OPT_WAIT_TIMEOUT_MS, OPT_MAX_REFINE, OPT_PROFILE = 1, 2, 3, 4, 5, 6
OPT_PRECOND, OPT_INNER_ITERATION, OPT_REFINE_TOL_SCALE, OPT_APPLY_PIPELINE, OPT_EXTRAP_ORDER = 7, 8, 9, 10, 11
OPT_ADAPTIVE_INNER = 12
OPT_RESIDENT = 13
OPT_PROJECT = 14
OPT_LEARNED_STEP = 15
PREC_FP64, PREC_MIXED = 0, 1
PRECOND_NONE, PRECOND_DIAG, PRECOND_FDM = 0, 1, 2
GUESS_ZERO, GUESS_EXTRAPOLATE, GUESS_LEARNED = 0, 1, 2

_lib = None


class SemError(RuntimeError):
    def __init__(self, status: int, where: str):
        L = load()
        msg = L.sem_last_error().decode(errors="replace")
        super().__init__(f"{where}: {L.sem_status_string(status).decode()} ({status}) {msg}")
        self.status = status


def load():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError(f"CUDA library not built: {LIB} (run schrodingersem_gb300.build.build())")
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        raise SemError(status, where)
