"""Loader for the oracle's threaded C restatement (oracle/dag_cholesky.c):
the tiled Cholesky and its solve, and the pivoted tiled LU.

TEST INFRASTRUCTURE ONLY: used by tests/ as a checker at larger sizes and by
bench.py's CPU-baseline leg.  The product library never loads it.

The C file is compiled with gcc into oracle/_build/ (by `build()` here, which
__graft_entry__.build() calls).  BLAS/LAPACK tile routines come from scipy's
cython_blas / cython_lapack capsules (LP64 Fortran ABI), so the same code runs
on x86-64 and aarch64 without BLAS headers.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "dag_cholesky.c")
LIB = os.path.join(BUILD, "liboracle_dag.so")

_lib = None


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread",
                               "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def _capsule_ptr(cap) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(cap, get_name(cap))


def set_blas_threads(n: int) -> bool:
    """Limit scipy's OpenBLAS to n threads (tile tasks run one per worker)."""
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__) + ".libs", "libscipy_openblas*.so*"))
    libs += glob.glob(os.path.join(os.path.dirname(scipy.__file__), ".dylibs", "*openblas*"))
    for path in libs:
        try:
            h = ctypes.CDLL(path)
        except OSError:
            continue
        for name in ("scipy_openblas_set_num_threads", "openblas_set_num_threads",
                     "scipy_openblas_set_num_threads64_"):
            fn = getattr(h, name, None)
            if fn is not None:
                fn.argtypes = [ctypes.c_int]
                fn(int(n))
                return True
    return False


def lib():
    global _lib
    if _lib is None:
        import scipy.linalg.cython_blas as cb
        import scipy.linalg.cython_lapack as cl
        L = ctypes.CDLL(build())
        L.oracle_set_blas.argtypes = [ctypes.c_void_p] * 4
        L.oracle_chol_tiled.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_solve_tiled.argtypes = [ctypes.c_char, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.oracle_set_getrf.argtypes = [ctypes.c_void_p]
        L.oracle_lu_tiled.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int]
        rc = L.oracle_set_blas(_capsule_ptr(cb.__pyx_capi__["dgemm"]),
                               _capsule_ptr(cb.__pyx_capi__["dtrsm"]),
                               _capsule_ptr(cb.__pyx_capi__["dsyrk"]),
                               _capsule_ptr(cl.__pyx_capi__["dpotrf"]))
        assert rc == 0
        assert L.oracle_set_getrf(_capsule_ptr(cl.__pyx_capi__["dgetrf"])) == 0
        _lib = L
    return _lib


def chol_tiled(A: np.ndarray, nb: int, uplo: str = 'U', nthreads: int = 1, inplace=False):
    """Threaded _chol!: returns (F, info) with F Fortran-ordered."""
    F = A if inplace else np.array(A, dtype=np.float64, order='F', copy=True)
    assert F.flags.f_contiguous and F.dtype == np.float64
    n = F.shape[0]
    info = lib().oracle_chol_tiled(uplo.encode(), n, nb, F.ctypes.data, n, nthreads)
    if info < 0:
        raise RuntimeError(f"oracle_chol_tiled failed: {info}")
    return F, int(info)


def ldiv_tiled(F: np.ndarray, uplo: str, B: np.ndarray, nb: int, nthreads: int = 1):
    """Threaded ldiv!(cholesky, B) in place on a Fortran-ordered B (n x nrhs)."""
    assert F.flags.f_contiguous and B.flags.f_contiguous
    n = F.shape[0]
    B2 = B.reshape(n, -1, order='F')
    rc = lib().oracle_solve_tiled(uplo.encode(), n, nb, F.ctypes.data, n, B2.shape[1],
                                  B2.ctypes.data, n, nthreads)
    if rc != 0:
        raise RuntimeError(f"oracle_solve_tiled failed: {rc}")
    return B


def lu_tiled(A: np.ndarray, nb: int, nthreads: int = 1, inplace=False):
    """Threaded lu!(A, RowMaximum()) (square A): returns (F, ipiv, info), F
    Fortran-ordered, ipiv the 1-based global pivots (int64)."""
    F = A if inplace else np.array(A, dtype=np.float64, order='F', copy=True)
    assert F.flags.f_contiguous and F.dtype == np.float64 and F.shape[0] == F.shape[1]
    n = F.shape[0]
    ipiv = np.zeros(max(n, 1), dtype=np.int32)
    info = lib().oracle_lu_tiled(n, nb, F.ctypes.data, n, ipiv.ctypes.data, nthreads)
    if info < 0:
        raise RuntimeError(f"oracle_lu_tiled failed: {info}")
    return F, ipiv[:n].astype(np.int64), int(info)
