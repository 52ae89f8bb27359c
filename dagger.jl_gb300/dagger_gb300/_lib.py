"""ctypes binding of libdaggergb300.so (include/dagger_gb300.h).

This is the Python counterpart of the `ccall` binding a Julia backend
would write: plain pointers, sizes and a stream.  The library must exist:
there is no CPU fallback, and a missing library raises at import of the
first compute call.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdaggergb300.so")

DG_OK = 0
DG_ERR_CUDA = -1000
DG_ERR_TIMEOUT = -1001
DG_ERR_NOMEM = -1002
DG_ERR_UNSUPPORTED = -1003
DG_ERR_NOCONVERGE = -1004
DG_ERR_STATE = -1005

DG_IN, DG_OUT, DG_INOUT = 1, 2, 3
DG_OP_POTRF, DG_OP_TRSM, DG_OP_SYRK, DG_OP_GEMM, DG_OP_COPY = 1, 2, 3, 4, 5

c_char, c_int, c_double, c_void_p = ctypes.c_char, ctypes.c_int, ctypes.c_double, ctypes.c_void_p
c_dp = ctypes.c_void_p  # device pointers are passed as integers


class DgTask(ctypes.Structure):
    _fields_ = [
        ("op", c_int),
        ("side", c_char), ("uplo", c_char), ("transa", c_char), ("transb", c_char),
        ("diag", c_char), ("trans", c_char),
        ("m", c_int), ("n", c_int), ("k", c_int),
        ("alpha", c_double), ("beta", c_double),
        ("a", c_void_p), ("lda", c_int),
        ("b", c_void_p), ("ldb", c_int),
        ("c", c_void_p), ("ldc", c_int),
        ("mode_a", c_int), ("mode_b", c_int), ("mode_c", c_int),
        ("info_offset", c_int),
    ]


class DgMixedStats(ctypes.Structure):
    _fields_ = [("n", c_int), ("nb", c_int), ("precision", c_int), ("info", c_int),
                ("retries", c_int), ("factor_ms", ctypes.c_float), ("norm_inf", c_double),
                ("device_bytes", ctypes.c_longlong), ("shift", c_double)]


class DgIrOpts(ctypes.Structure):
    _fields_ = [("tol", c_double), ("max_iter", c_int), ("gmres", c_int), ("restart", c_int),
                ("gmres_inner_tol", c_double)]


class DgIrReport(ctypes.Structure):
    _fields_ = [("iterations", c_int), ("gmres_iterations", c_int), ("used_gmres", c_int),
                ("converged", c_int), ("backward_error", c_double), ("solve_ms", ctypes.c_float)]


DG_PREC = {"bf16": 1, "bf16x3": 3, "bf16x6": 6, "fp8": 8, "fp16": 11, "fp16x3": 13, "fp32": 32}

# name -> (restype, argtypes); every symbol include/dagger_gb300.h declares.
SIGNATURES = {
    "dg_version": (ctypes.c_char_p, []),
    "dg_last_error": (ctypes.c_char_p, []),
    "dg_finalize": (c_int, []),
    "dg_release_memory": (c_int, []),
    "dg_kernel_launches": (ctypes.c_longlong, []),
    "dg_set_device": (c_int, [c_int]),
    "dg_device_alloc": (c_int, [ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    "dg_device_free": (c_int, [c_void_p]),
    "dg_host_alloc": (c_int, [ctypes.c_size_t, ctypes.POINTER(c_void_p)]),
    "dg_host_free": (c_int, [c_void_p]),
    "dg_copy": (c_int, [c_void_p, c_void_p, ctypes.c_size_t, c_int, c_void_p]),
    "dg_stream_create": (c_int, [ctypes.POINTER(c_void_p)]),
    "dg_stream_destroy": (c_int, [c_void_p]),
    "dg_stream_synchronize": (c_int, [c_void_p]),
    "dg_potrf": (c_int, [c_char, c_int, c_dp, c_int, ctypes.POINTER(c_int), c_void_p]),
    "dg_potrf_async": (c_int, [c_char, c_int, c_dp, c_int, c_dp, c_void_p]),
    "dg_trsm": (c_int, [c_char, c_char, c_char, c_char, c_int, c_int, c_double, c_dp, c_int,
                        c_dp, c_int, c_void_p]),
    "dg_syrk": (c_int, [c_char, c_char, c_int, c_int, c_double, c_dp, c_int, c_double, c_dp,
                        c_int, c_void_p]),
    "dg_gemm": (c_int, [c_char, c_char, c_int, c_int, c_int, c_double, c_dp, c_int, c_dp, c_int,
                        c_double, c_dp, c_int, c_void_p]),
    "dg_trsv": (c_int, [c_char, c_char, c_char, c_int, c_dp, c_int, c_dp, c_void_p]),
    "dg_gemv": (c_int, [c_char, c_int, c_int, c_double, c_dp, c_int, c_dp, c_double, c_dp,
                        c_void_p]),
    "dg_region_create": (c_void_p, []),
    "dg_region_add": (c_int, [c_void_p, ctypes.POINTER(DgTask)]),
    "dg_region_stats": (c_int, [c_void_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "dg_region_edges": (c_int, [c_void_p, ctypes.POINTER(c_int), c_int]),
    "dg_region_run": (c_int, [c_void_p, c_int, c_int, c_void_p]),
    "dg_region_destroy": (None, [c_void_p]),
    "dg_cholesky_tiled": (c_int, [c_char, c_int, c_int, c_void_p, c_void_p]),
    "dg_cholesky_solve_tiled": (c_int, [c_char, c_int, c_int, c_void_p, c_int, c_void_p,
                                        c_void_p]),
    "dg_cholesky_tiled_winv": (c_int, [c_char, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    "dg_cholesky_tiled_host": (c_int, [c_char, c_int, c_int, c_void_p, ctypes.c_longlong, c_void_p,
                                       c_void_p, c_void_p]),
    "dg_cholesky_solve_tiled_winv": (c_int, [c_char, c_int, c_int, c_void_p, c_void_p, c_int,
                                             c_void_p, c_void_p]),
    "dg_gemm_tiled": (c_int, [c_char, c_char, c_int, c_int, c_int, c_int, c_double, c_void_p,
                              c_void_p, c_double, c_void_p, c_void_p]),
    "dg_syrk_tiled": (c_int, [c_char, c_int, c_int, c_int, c_double, c_void_p, c_double,
                              c_void_p, c_void_p]),
    "dg_getrf": (c_int, [c_int, c_int, c_dp, c_int, c_void_p, ctypes.POINTER(c_int), c_void_p]),
    "dg_lu_tiled": (c_int, [c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "dg_lu_solve_tiled": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "dg_set_f64_engine": (c_int, [c_int]),
    "dg_get_f64_engine": (c_int, []),
    "dg_ishermitian_tiled": (c_int, [c_int, c_int, c_void_p, c_void_p]),
    "dg_chkfinite_tiled": (c_int, [c_int, c_int, c_void_p, c_void_p]),
    "dg_chkfinite_tiled_mn": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    "dg_copy_reblock": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_int, c_int, c_void_p,
                                c_void_p]),
    "dg_probe_fp64_fma_tflops": (c_int, [c_int, ctypes.POINTER(c_double), c_void_p]),
    "dg_mixed_factor": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_void_p, c_int,
                                c_void_p]),
    "dg_mixed_factor_ex": (c_int, [ctypes.POINTER(c_void_p), c_int, c_int, c_void_p, c_int,
                                   c_double, c_void_p]),
    "dg_mixed_solve": (c_int, [c_void_p, c_int, c_dp, c_int, c_dp, c_int,
                               ctypes.POINTER(DgIrOpts), ctypes.POINTER(DgIrReport), c_void_p]),
    "dg_mixed_info": (c_int, [c_void_p, ctypes.POINTER(DgMixedStats)]),
    "dg_mixed_destroy": (None, [c_void_p]),
    "dg_gemm_tc_tn": (c_int, [c_int, c_int, c_int, c_int, c_int, c_dp, c_dp, c_int, c_dp, c_dp,
                              c_int, ctypes.c_float, ctypes.c_float, c_dp, c_int, c_int, c_dp,
                              c_void_p]),
    "dg_gemm_f32_tc_tn": (c_int, [c_int, c_int, c_int, ctypes.c_float, c_dp, c_int, c_dp, c_int,
                                  ctypes.c_float, c_dp, c_int, c_void_p]),
    "dg_gemm_f8_tc_tn": (c_int, [c_int, c_int, c_int, ctypes.c_float, c_dp, c_int, c_dp, c_int,
                                 ctypes.c_float, c_dp, c_int, c_void_p]),
    "dg_potrf_inv_f32": (c_int, [c_int, c_dp, c_int, c_dp, c_int, ctypes.POINTER(c_int),
                                 c_void_p]),
    "dg_gemm_f64_emulated_tn": (c_int, [c_int, c_int, c_int, c_double, c_void_p, c_int, c_void_p,
                                        c_int, c_double, c_void_p, c_int, c_void_p]),
    "dg_f64_slices": (c_int, [c_int, c_int, c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                              c_void_p, c_int, c_void_p, c_void_p]),
    "dg_gemm_f64_slices": (c_int, [c_int, c_int, c_int, c_double, c_void_p, c_int, c_void_p,
                                   c_void_p, c_int, c_void_p, c_double, c_void_p, c_int, c_void_p,
                                   c_void_p]),
    "dg_batched_potrs": (c_int, [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int), c_void_p,
                                 c_void_p, c_void_p, c_int, c_double, c_int,
                                 ctypes.POINTER(c_int), c_int, ctypes.POINTER(c_int),
                                 ctypes.POINTER(c_double), ctypes.POINTER(ctypes.c_float),
                                 c_void_p]),
    "dg_batched_potrs_noalloc": (c_int, [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                         c_void_p, c_void_p, c_void_p, c_int, c_double, c_int,
                                         ctypes.POINTER(c_int), c_int, ctypes.POINTER(c_int),
                                         ctypes.POINTER(c_double), c_void_p]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """Loads the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB_PATH):
                    raise RuntimeError(
                        f"{LIB_PATH} is missing: build it with dagger.jl_gb300/build.py "
                        "(there is no CPU fallback)")
                L = ctypes.CDLL(LIB_PATH)
                for name, (res, args) in SIGNATURES.items():
                    fn = getattr(L, name)
                    fn.restype = res
                    fn.argtypes = args
                _lib = L
    return _lib


def last_error() -> str:
    return lib().dg_last_error().decode()


class PosDefException(Exception):
    """LinearAlgebra.PosDefException(info): the leading minor of order info
    is not positive definite."""

    def __init__(self, info: int):
        super().__init__(f"matrix is not positive definite; Cholesky factorization failed (info={info})")
        self.info = info


class SingularException(Exception):
    """LinearAlgebra.SingularException(info): U[info, info] of an LU is
    exactly zero."""

    def __init__(self, info: int):
        super().__init__(f"SingularException({info})")
        self.info = info


class DaggerGB300Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libdaggergb300 error {code}: {msg}")
        self.code = code


def check(rc: int, *, posdef: bool = False) -> int:
    """Maps a status to Python: >0 info (PosDefException when posdef),
    -i invalid argument i (ValueError), <= -1000 library error."""
    if rc == 0:
        return 0
    if rc > 0:
        if posdef:
            raise PosDefException(rc)
        return rc
    if rc > -1000:
        raise ValueError(f"invalid argument {-rc}: {last_error()}")
    if rc == DG_ERR_NOMEM:
        raise MemoryError(last_error())
    raise DaggerGB300Error(rc, last_error())


def ch(c: str) -> bytes:
    return c.encode() if isinstance(c, str) else c
