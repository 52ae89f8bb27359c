"""The oracle's restatement of gemm_dagger! / syrk_dagger! (src/array/mul.jl)
against dense FP64 products: the tile loops must reproduce alpha op(A) op(B)
+ beta C, and syrk_dagger! a fully symmetric C (copytri!)."""
import numpy as np
import pytest

from oracle import tiled as o


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,nb", [(70, 50, 90, 32), (64, 64, 64, 16), (5, 7, 3, 4)])
def test_gemm_dagger_matches_dense(ta, tb, m, n, k, nb):
    r = np.random.default_rng(m * n + k)
    A = r.standard_normal((m, k) if ta == "N" else (k, m))
    B = r.standard_normal((k, n) if tb == "N" else (n, k))
    C = r.standard_normal((m, n))
    got = o.gemm_dagger(C, ta, tb, A, B, 0.5, -1.5, nb)
    opA = A if ta == "N" else A.T
    opB = B if tb == "N" else B.T
    ref = 0.5 * opA @ opB - 1.5 * C
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,k,nb", [(70, 90, 32), (64, 20, 16), (9, 5, 4)])
def test_syrk_dagger_matches_dense(trans, n, k, nb):
    r = np.random.default_rng(n + k)
    A = r.standard_normal((n, k) if trans == "N" else (k, n))
    S = r.standard_normal((n, n))
    C = S + S.T
    got = o.syrk_dagger(C, trans, A, 2.0, 0.5, nb)
    opA = A if trans == "N" else A.T
    ref = 2.0 * opA @ opA.T + 0.5 * C
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.array_equal(got, got.T)
