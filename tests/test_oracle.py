"""The oracle itself (CPU, no GPU): pinned to FP64 LAPACK through the golden
fixtures and the reference's own test recipes, and its threaded C form
checked bit-for-bit against the Python restatement."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SQRT_EPS = np.sqrt(np.finfo(float).eps)


def _rel(x, y):
    return np.abs(x - y).max() / np.abs(y).max()


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                                         if not os.path.basename(p).startswith("lu_")),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_golden_fixture(path):
    from oracle import tiled as o
    g = np.load(path)
    A, nb, uplo = g["A"], int(g["nb"]), str(g["uplo"])
    if os.path.basename(path).startswith("chol"):
        F, info = o.chol_tiled(A, nb, uplo)
        assert info == 0
        T = o.triangle(F, uplo)
        # oracle reproduces its stored tiled factor (any BLAS build: 1e-14) ...
        assert _rel(T, g["tiled"]) <= 1e-14
        # ... which agrees with FP64 LAPACK (the reference tests' comparison;
        # the M M' recipe of test/datadeps.jl has kappa ~ 4e7, so it is held
        # to that test's isapprox tolerance, sqrt(eps))
        tol = SQRT_EPS if "datadeps" in path else 1e-13
        assert _rel(g["tiled"], g["lapack"]) <= tol
        assert o.factor_residual(A, F, uplo) <= 1e-14
    else:
        B = g["B"]
        F, _ = o.chol_tiled(A, nb, uplo)
        X = np.array(B, order='F', copy=True)
        o.ldiv_cholesky(F, uplo, X, nb)
        assert _rel(X, g["tiled"]) <= 1e-14
        assert _rel(g["tiled"], g["lapack"]) <= 1e-12


def test_reference_recipe_cholesky():
    """test/array/linalg/cholesky.jl:8-35: factor ≈ stdlib (rtol sqrt(eps))."""
    from oracle import tiled as o
    for uplo in "UL":
        A = np.random.default_rng(0).random((128, 128))
        A = np.asfortranarray(A @ A.T + 128 * np.eye(128))
        F, info = o.chol_tiled(A, 32, uplo)
        Fl, _ = o.lapack_factor(A, uplo)
        assert info == 0 and _rel(o.triangle(F, uplo), Fl) <= SQRT_EPS
        assert o.ishermitian_tiled(A, 32)
    assert not o.ishermitian_tiled(np.random.default_rng(1).random((32, 32)), 4)


def test_reference_recipe_datadeps_lower():
    """test/datadeps.jl:946-984: hand-spawned lower DAG ≈ LAPACK.potrf!('L')."""
    from oracle import tiled as o
    M = np.random.default_rng(2).random((1000, 1000))
    M = np.asfortranarray(M @ M.T)
    F, info = o.chol_tiled(M, 100, 'L')
    Fl, _ = o.lapack_factor(M, 'L')
    assert info == 0 and _rel(np.tril(F), Fl) <= SQRT_EPS


def test_reference_recipe_mpi():
    """test/mpi_cholesky.jl: both errors < 1e-12."""
    from oracle import tiled as o
    A = np.random.default_rng(42).random((64, 64))
    A = np.asfortranarray(A @ A.T + 64 * np.eye(64))
    F, _ = o.chol_tiled(A, 16, 'U')
    U = np.triu(F)
    Uref, _ = o.lapack_factor(A, 'U')
    assert np.linalg.norm(U - Uref) / np.linalg.norm(Uref) < 1e-12
    assert np.linalg.norm(U.T @ U - A) / np.linalg.norm(A) < 1e-12


@pytest.mark.parametrize("uplo", "UL")
def test_reference_recipe_solve(uplo):
    """test/array/linalg/solve.jl:46-71: matrix and vector RHS ≈ stdlib."""
    from oracle import tiled as o
    rng = np.random.default_rng(4)
    A = rng.random((128, 128))
    A = np.asfortranarray(A.T @ A + np.eye(128))
    B = np.asfortranarray(rng.random((128, 128)))
    F, _ = o.chol_tiled(A, 64, uplo)
    X = B.copy(order='F')
    o.ldiv_cholesky(F, uplo, X, 64)
    assert _rel(X, o.lapack_solve(A, B, uplo)) <= SQRT_EPS
    b = rng.random(128)
    x = b.copy()
    o.ldiv_cholesky(F, uplo, x, 64)
    assert _rel(x, o.lapack_solve(A, b[:, None], uplo)[:, 0]) <= 1e-10


@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NT")
def test_trsm_tiled_all_branches(side, uplo, trans):
    """Every branch of Dagger.trsm! (trsm.jl:89-189) against a dense solve."""
    from oracle import tiled as o
    rng = np.random.default_rng(8)
    n, nb = 70, 16
    A = np.asfortranarray(rng.standard_normal((n, n)) + n * np.eye(n))
    B = np.asfortranarray(rng.standard_normal((n, n)))
    X = B.copy(order='F')
    o.trsm_tiled(side, uplo, trans, 'N', 1.0, A, X, nb)
    T = np.triu(A) if uplo == 'U' else np.tril(A)
    op = T.T if trans == 'T' else T
    ref = np.linalg.solve(op, B) if side == 'L' else np.linalg.solve(op.T, B.T).T
    assert _rel(X, ref) <= 1e-13


@pytest.mark.parametrize("uplo", "UL")
def test_not_posdef_info(uplo):
    from oracle import tiled as o
    A = o.spd_uniform(128, 5)
    A[70, 70] = -1.0
    _, info = o.chol_tiled(A, 32, uplo)
    _, info_l = o.lapack_factor(A, uplo)
    assert info == info_l == 71
    with pytest.raises(o.PosDefException):
        o.cholesky(A, 32, uplo)


@pytest.mark.parametrize("uplo", "UL")
def test_threaded_c_oracle_is_bit_identical(uplo):
    """The threaded C restatement runs the same BLAS calls in a dependency
    order the datadeps rules allow: identical bits to the Python loop."""
    from oracle import native, tiled as o
    native.set_blas_threads(1)
    for n, nb in [(130, 32), (1000, 128)]:
        A = o.spd_uniform(n, n)
        F1, i1 = o.chol_tiled(A, nb, uplo)
        F2, i2 = native.chol_tiled(A, nb, uplo, nthreads=4)
        assert i1 == i2 == 0
        assert np.array_equal(o.triangle(F1, uplo), o.triangle(F2, uplo))
        B = o.rhs_normal(n, 7, 1)
        X1, X2 = B.copy(order='F'), B.copy(order='F')
        o.ldiv_cholesky(F1, uplo, X1, nb)
        native.ldiv_tiled(F2, uplo, X2, nb, 4)
        assert np.array_equal(X1, X2)


def test_datadeps_edges_are_the_classic_tile_dependencies():
    """The datadeps rules yield POTRF(k) <- SYRK(k-1); TRSM(k,n) <- POTRF(k),
    GEMM(k-1 on k,n); SYRK <- TRSM + previous SYRK; GEMM <- two TRSMs + the
    previous GEMM on the same tile."""
    from oracle.tiled import chol_tasks, datadeps_edges
    tasks = chol_tasks(4, 'U')
    preds = datadeps_edges(tasks)
    index = {(k, tuple(r), tuple(w)): i for i, (k, r, w) in enumerate(tasks)}
    potrf1 = index[('potrf', (), ((1, 1),))]
    syrk01 = index[('syrk', ((0, 1),), ((1, 1),))]
    assert preds[potrf1] == {syrk01}
    gemm_1_23 = index[('gemm', ((1, 2), (1, 3)), ((2, 3),))]
    trsm_12 = index[('trsm', ((1, 1),), ((1, 2),))]
    trsm_13 = index[('trsm', ((1, 1),), ((1, 3),))]
    gemm_0_23 = index[('gemm', ((0, 2), (0, 3)), ((2, 3),))]
    assert preds[gemm_1_23] == {trsm_12, trsm_13, gemm_0_23}
