"""The oracle's restatement of lu!(A, RowMaximum()) / lu!(A, NoPivot()) and
ldiv!(F::LU, B) (src/array/lu.jl, linalg.jl:264-308), pinned against untiled
FP64 LAPACK (dgetrf / dgetrs through scipy) with the recipes and tolerances of
test/array/linalg/lu.jl, and against the committed golden fixtures."""
import os

import numpy as np
import pytest
from scipy.linalg import lapack

from oracle import lu as o

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def lapack_lu(A):
    lu, piv, info = lapack.dgetrf(np.asfortranarray(A))
    return lu, piv.astype(np.int64) + 1, int(info)


@pytest.mark.parametrize("m,n,nb", [(128, 128, 64), (128, 128, 32), (200, 200, 64),
                                    (130, 130, 32), (300, 200, 64), (200, 300, 64),
                                    (64, 64, 16), (37, 37, 8)])
def test_rowmaximum_matches_lapack(m, n, nb):
    A = o.rand_uniform(m, n, m * 1000 + n + nb)
    F, ipiv, info = o.lu_rowmaximum(A, nb)
    Fl, pl, il = lapack_lu(A)
    assert info == il == 0
    # the same row-by-row partial pivoting: identical pivots
    assert np.array_equal(ipiv, pl)
    assert np.linalg.norm(F - Fl) <= 1e-12 * np.linalg.norm(Fl)
    # test/array/linalg/lu.jl: P*A ≈ L*U rtol 1e-12
    assert o.lu_residual(A, F, ipiv) <= 1e-12


def test_rowmaximum_reference_recipe_128_64():
    """test/array/linalg/lu.jl:17-42: rand(128, 128), Blocks(64, 64), the
    factorization and A \\ b."""
    A = o.rand_uniform(128, 128, 1)
    F, ipiv, info = o.lu(A, 64)
    L, U = o.factors_LU(F)
    P = np.eye(128)[o.permutation(ipiv, 128)]
    # Julia's isapprox is normwise: norm(x - y) <= rtol * max(norm(x), norm(y))
    assert np.linalg.norm(P @ A - L @ U) <= 1e-12 * np.linalg.norm(P @ A)
    assert np.allclose(P.T @ P, np.eye(128))
    assert np.array_equal(U, np.triu(U)) and np.array_equal(L, np.tril(L))
    b = np.random.default_rng(2).random(128)
    x = o.ldiv_lu(F, ipiv, b.copy(), 64)
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)


def test_nopivot_matches_unpivoted_lapack():
    """generic_lufact! + TRSMs on a diagonally dominant matrix, where LAPACK's
    partial pivoting keeps every pivot on the diagonal."""
    A = o.rand_uniform(150, 150, 3)
    A[np.diag_indices(150)] += 150.0
    F, ipiv, info = o.lu_nopivot(A, 32)
    Fl, pl, il = lapack_lu(A)
    assert np.array_equal(pl, np.arange(1, 151))
    assert info == 0
    assert np.array_equal(ipiv, np.arange(1, 151))
    assert np.linalg.norm(F - Fl) <= 1e-13 * np.linalg.norm(Fl)


def test_nopivot_reference_tolerance():
    """test/array/linalg/lu.jl: NoPivot P*A ≈ L*U to rtol 1e-7 on rand(128, 128)."""
    A = o.rand_uniform(128, 128, 11)
    F, ipiv, info = o.lu(A, 64, pivot='nopivot')
    assert info == 0
    assert o.lu_residual(A, F, ipiv) <= 1e-7


def test_singular_ones():
    """test/array/linalg/lu.jl:100: lu(ones(128, 128)) throws SingularException."""
    A = np.asfortranarray(np.ones((128, 128)))
    with pytest.raises(o.SingularException) as e:
        o.lu(A, 64)
    _, _, il = lapack_lu(A)
    assert e.value.info == il == 2
    F, ipiv, info = o.lu(A, 64, allowsingular=True)
    assert info == 2


def test_info_first_zero_pivot_matches_lapack():
    A = o.rand_uniform(96, 96, 4)
    A[:, 70] = 0.0                       # column 71 has no pivot
    _, _, info = o.lu_rowmaximum(A, 32)
    _, _, il = lapack_lu(A)
    assert info == il == 71


@pytest.mark.parametrize("nrhs", [1, 5, 40])
def test_ldiv_matches_lapack(nrhs):
    n, nb = 160, 32
    A = o.rand_uniform(n, n, 8)
    B = np.asfortranarray(np.random.default_rng(9).standard_normal((n, nrhs)))
    F, ipiv, _ = o.lu_rowmaximum(A, nb)
    X = o.ldiv_lu(F, ipiv, B.copy(), nb)
    lu, piv, _ = lapack.dgetrf(A)
    Xl, _ = lapack.dgetrs(lu, piv, B)
    assert np.abs(X - Xl).max() <= 1e-10 * np.abs(Xl).max()
    R = B - A @ X
    berr = np.abs(R).max(0) / (np.abs(A).sum(1).max() * np.abs(X).max(0) + np.abs(B).max(0))
    assert berr.max() <= 1e-14


def test_apply_ipiv_rows_is_the_permutation():
    n, nb = 100, 16
    A = o.rand_uniform(n, n, 12)
    _, ipiv, _ = o.lu_rowmaximum(A, nb)
    B = np.asfortranarray(np.arange(n * 3, dtype=np.float64).reshape(n, 3))
    got = o.apply_ipiv_rows(ipiv, B.copy(order='F'), nb)
    assert np.array_equal(got, B[o.permutation(ipiv, n), :])


@pytest.mark.parametrize("n,nb", [(128, 64), (130, 32), (600, 128), (1024, 256)])
def test_threaded_c_lu_matches_python_oracle(n, nb):
    """oracle/dag_cholesky.c's threaded lu!(A, RowMaximum()) (the benchmark's
    CPU baseline) against the Python restatement and LAPACK."""
    from oracle import native
    A = o.rand_uniform(n, n, n + nb)
    F, ipiv, info = native.lu_tiled(A, nb, nthreads=4)
    F0, p0, i0 = o.lu_rowmaximum(A, nb)
    assert info == i0 == 0
    assert np.array_equal(ipiv, p0)
    assert np.linalg.norm(F - F0) <= 1e-14 * np.linalg.norm(F0)
    Z = np.asfortranarray(np.ones((128, 128)))
    assert native.lu_tiled(Z, 64, nthreads=4)[2] == 2


@pytest.mark.parametrize("seed", range(6))
def test_row_list_equals_pairwise_swaps(seed):
    """The CUDA path applies a panel's interchanges to the other block columns
    as one (destination, source) row list; the reference swaps tile pair by
    tile pair in pivot order (swaprows_trail!).  Both must move the same rows,
    including pivots that hit the same row twice and pivots inside the panel."""
    r = np.random.default_rng(seed)
    nb, mt, k = 16, 5, 1
    m = nb * mt
    row0 = k * nb
    ipk = np.empty(nb, dtype=np.int64)
    for p in range(nb):                       # LAPACK form: ipiv[p] >= row0 + p + 1
        lo = row0 + p
        ipk[p] = (lo if r.random() < 0.2 else r.integers(lo, m)) + 1
    if seed % 2:                              # a row chosen twice
        ipk[nb - 1] = ipk[nb // 2] = max(ipk[nb // 2], row0 + nb)
    X = np.asfortranarray(r.standard_normal((m, 3)))
    ref = X.copy(order='F')
    for i in range(k, mt):
        o.swaprows_trail(ref[row0:row0 + nb, :], ref[i * nb:(i + 1) * nb, :], ipk, i, nb)
    got = X[row0:, :].copy()
    o.apply_row_list(o.panel_row_list(ipk, row0), got)
    assert np.array_equal(got, ref[row0:, :])
    assert len(o.panel_row_list(ipk, row0)) <= 2 * nb


@pytest.mark.parametrize("name", ["lu_rowmax_128_64", "lu_rowmax_ragged_200x150_64",
                                  "lu_nopiv_96_32", "lu_solve_160_32_r5"])
def test_golden_fixtures(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    nb = int(z["nb"])
    A = np.asfortranarray(z["A"])
    if "B" in z:
        F, ipiv, _ = o.lu_rowmaximum(A, nb)
        X = o.ldiv_lu(F, ipiv, np.asfortranarray(z["B"]).copy(), nb)
        assert np.abs(X - z["tiled"]).max() <= 1e-12 * np.abs(z["tiled"]).max()
        assert np.abs(X - z["lapack"]).max() <= 1e-10 * np.abs(z["lapack"]).max()
        return
    pivot = str(z["pivot"])
    F, ipiv, info = o.lu(A, nb, pivot=pivot)
    assert np.array_equal(ipiv, z["ipiv"])
    assert np.linalg.norm(F - z["tiled"]) <= 1e-13 * np.linalg.norm(z["tiled"])
    if "lapack" in z:
        assert np.linalg.norm(F - z["lapack"]) <= 1e-12 * np.linalg.norm(z["lapack"])
