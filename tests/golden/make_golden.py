"""Generates the small golden fixtures under tests/golden/.

The reference ships no golden vectors for this path and cannot be run here
(it is Julia), so the fixtures pin the oracle to FP64 LAPACK: for seeded
inputs built with the recipes of the reference's tests they store the input,
the LAPACK factor / solution, and the oracle's tiled factor / solution.

    python tests/golden/make_golden.py

Recipes (paths within JuliaParallel/Dagger.jl):
  chol_mpi_U_64_16      test/mpi_cholesky.jl: rand(64,64); A*A'; diag += 64; Blocks(16,16)
  chol_linalg_U_128_32  test/array/linalg/cholesky.jl: rand(128,128); A*A'; diag += 128
  chol_datadeps_L_200_50   test/datadeps.jl:946-984 (lower DAG; 200 x 200, nb 50)
  chol_ragged_U_130_32  a ragged tiling (130 = 4*32 + 2)
  solve_U_128_64_r5     test/array/linalg/solve.jl: A'A + I, DMatrix RHS
  solve_L_96_32_vec     vector right-hand side (trsv! path)
  lu_rowmax_128_64      test/array/linalg/lu.jl: rand(128, 128), Blocks(64, 64), RowMaximum
  lu_rowmax_ragged_200x150_64  a rectangular, ragged tiling
  lu_nopiv_96_32        NoPivot on a diagonally dominant rand(96, 96) + 96 I
  lu_solve_160_32_r5    lu(A) \\ B with 5 right-hand sides
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import lu as olu  # noqa: E402
from oracle import tiled as o  # noqa: E402


def rand_spd_aat(n, seed, shift):
    rng = np.random.default_rng(seed)
    A = rng.random((n, n))
    A = A @ A.T
    A[np.diag_indices(n)] += shift
    return np.asfortranarray(A)


def main():
    cases = {}

    def factor_case(name, A, nb, uplo):
        F, info = o.chol_tiled(A, nb, uplo)
        assert info == 0
        Fl, _ = o.lapack_factor(A, uplo)
        cases[name] = dict(A=A, nb=np.int64(nb), uplo=np.array(uplo),
                           tiled=o.triangle(F, uplo), lapack=Fl)

    factor_case("chol_mpi_U_64_16", rand_spd_aat(64, 42, 64), 16, 'U')
    factor_case("chol_linalg_U_128_32", rand_spd_aat(128, 1, 128), 32, 'U')
    rng = np.random.default_rng(5)
    M = rng.random((200, 200))
    factor_case("chol_datadeps_L_200_50", np.asfortranarray(M @ M.T), 50, "L")
    factor_case("chol_ragged_U_130_32", o.spd_uniform(130, 7), 32, 'U')

    def solve_case(name, A, B, nb, uplo):
        F, info = o.chol_tiled(A, nb, uplo)
        assert info == 0
        X = np.array(B, order='F', copy=True)
        o.ldiv_cholesky(F, uplo, X, nb)
        ref = o.lapack_solve(A, B.reshape(B.shape[0], -1), uplo)
        cases[name] = dict(A=A, B=B, nb=np.int64(nb), uplo=np.array(uplo), tiled=X,
                           lapack=ref.reshape(B.shape))

    rng = np.random.default_rng(9)
    A = rng.random((128, 128))
    solve_case("solve_U_128_64_r5", np.asfortranarray(A.T @ A + np.eye(128)),
               np.asfortranarray(rng.random((128, 5))), 64, 'U')
    A = o.spd_uniform(96, 3)
    solve_case("solve_L_96_32_vec", A, rng.standard_normal(96), 32, 'L')

    from scipy.linalg import lapack

    def lu_case(name, A, nb, pivot):
        F, ipiv, info = olu.lu(A, nb, pivot=pivot)
        assert info == 0
        d = dict(A=A, nb=np.int64(nb), pivot=np.array(pivot), tiled=F, ipiv=ipiv)
        if pivot == 'rowmaximum' or np.all(lapack.dgetrf(A)[1] == np.arange(min(A.shape))):
            d["lapack"] = lapack.dgetrf(A)[0]
        cases[name] = d

    lu_case("lu_rowmax_128_64", olu.rand_uniform(128, 128, 21), 64, 'rowmaximum')
    lu_case("lu_rowmax_ragged_200x150_64", olu.rand_uniform(200, 150, 22), 64, 'rowmaximum')
    A = olu.rand_uniform(96, 96, 23)
    A[np.diag_indices(96)] += 96.0
    lu_case("lu_nopiv_96_32", A, 32, 'nopivot')
    A = olu.rand_uniform(160, 160, 24)
    B = np.asfortranarray(np.random.default_rng(25).standard_normal((160, 5)))
    F, ipiv, _ = olu.lu(A, 32)
    X = olu.ldiv_lu(F, ipiv, B.copy(), 32)
    lu, piv, _ = lapack.dgetrf(A)
    cases["lu_solve_160_32_r5"] = dict(A=A, B=B, nb=np.int64(32), tiled=X,
                                       lapack=lapack.dgetrs(lu, piv, B)[0])

    for name, arrs in cases.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
    print("wrote", len(cases), "fixtures")


if __name__ == "__main__":
    main()
