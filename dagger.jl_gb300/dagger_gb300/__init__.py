"""dagger_gb300: GB300-native tiled Cholesky factor-and-solve behind
Dagger.jl's API for that path.

The compute runs in libdaggergb300.so (hand-written sm_103a CUDA kernels
behind the C ABI of include/dagger_gb300.h); this package is the host-side
mirror of the reference's interface (DArray/Blocks, cholesky, cholesky!,
ldiv!, ishermitian, spawn_datadeps with In/Out/InOut and the BLAS/LAPACK
tile calls).
"""
from ._lib import DaggerGB300Error, PosDefException, SingularException, lib
from .darray import Blocks, DArray, distribute
from .datadeps import In, InOut, Out, copyto_, spawn, spawn_datadeps
from .linalg import (Cholesky, chkfinite, cholesky, cholesky_, cholesky_distribute, copy_reblock,
                     gemm_, gemm_dagger_,
                     matmul, mul_, syrk_dagger_, gemm_f64_emulated_tn, gemv_,
                     get_f64_engine, getrf_, ishermitian, issymmetric, LU, ldiv, ldiv_, lu, lu_,
                     potrf_, set_f64_engine, syrk_, tile_local_info, trsm_, trsv_)
from .mixed import MixedCholesky, cholesky_mixed

__all__ = [
    "Blocks", "DArray", "distribute", "Cholesky", "cholesky", "cholesky_", "cholesky_distribute",
    "ldiv_", "gemm_dagger_", "syrk_dagger_", "mul_", "matmul",
    "ishermitian", "issymmetric", "potrf_", "trsm_", "syrk_", "gemm_", "trsv_", "gemv_",
    "gemm_f64_emulated_tn", "set_f64_engine", "get_f64_engine", "spawn_datadeps", "spawn", "In", "Out", "InOut", "copyto_", "PosDefException",
    "DaggerGB300Error", "lib", "LU", "lu", "lu_", "ldiv", "getrf_", "SingularException",
    "chkfinite", "copy_reblock", "tile_local_info", "MixedCholesky", "cholesky_mixed",
]
