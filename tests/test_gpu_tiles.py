"""Tile calls through the C ABI vs the oracle's BLAS/LAPACK tile kernels.

Each case runs the same seeded inputs through dg_gemm / dg_syrk / dg_trsm /
dg_potrf (via the dagger_gb300 mirrors of BLAS.gemm!, syrk!, trsm!,
LAPACK.potrf!) and through scipy's BLAS/LAPACK (the oracle's tile kernels),
on both FP64 engines (DMMA and DFMA).  Tolerance: FP64_RTOL = 1e-13 relative
to the largest entry of the reference result.
"""
import numpy as np
import pytest

from helpers import FP64_RTOL, dev_f, host_f, rel_err

pytestmark = pytest.mark.gpu

ENGINES = [0, 1]


@pytest.fixture(params=ENGINES, ids=["dfma", "dmma"])
def engine(request):
    import dagger_gb300 as d
    old = d.lib().dg_set_f64_engine(request.param)
    yield request.param
    d.lib().dg_set_f64_engine(old)


def _rng(seed):
    return np.random.default_rng(seed)


@pytest.mark.parametrize("ta", "NT")
@pytest.mark.parametrize("tb", "NT")
@pytest.mark.parametrize("m,n,k", [(64, 64, 64), (1, 1, 1), (70, 33, 129), (128, 200, 17),
                                   (257, 130, 300), (5, 300, 0)])
def test_gemm(engine, ta, tb, m, n, k):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = _rng(m * 1000 + n * 10 + k)
    A = np.asfortranarray(r.standard_normal((m, k) if ta == 'N' else (k, m)))
    B = np.asfortranarray(r.standard_normal((k, n) if tb == 'N' else (n, k)))
    C = np.asfortranarray(r.standard_normal((m, n)))
    ref = o._gemm(ta, tb, -1.0, A, B, 0.75, C.copy(order='F'))
    Cd = dev_f(C)
    d.gemm_(ta, tb, -1.0, dev_f(A), dev_f(B), 0.75, Cd)
    assert rel_err(host_f(Cd), ref) <= FP64_RTOL


def test_gemm_beta_zero_ignores_nan(engine):
    import dagger_gb300 as d
    r = _rng(5)
    A = np.asfortranarray(r.standard_normal((40, 30)))
    B = np.asfortranarray(r.standard_normal((30, 50)))
    C = np.full((40, 50), np.nan, order='F')
    Cd = dev_f(C)
    d.gemm_('N', 'N', 1.0, dev_f(A), dev_f(B), 0.0, Cd)
    assert rel_err(host_f(Cd), A @ B) <= FP64_RTOL


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NT")
@pytest.mark.parametrize("n,k", [(64, 64), (100, 37), (1, 5), (300, 257)])
def test_syrk(engine, uplo, trans, n, k):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = _rng(n * 7 + k)
    A = np.asfortranarray(r.standard_normal((n, k) if trans == 'N' else (k, n)))
    C = np.asfortranarray(r.standard_normal((n, n)))
    ref = o._syrk(uplo, trans, -1.0, A, 1.0, C.copy(order='F'))
    Cd = dev_f(C)
    d.syrk_(uplo, trans, -1.0, dev_f(A), 1.0, Cd)
    out = host_f(Cd)
    assert rel_err(out, ref) <= FP64_RTOL
    # the other triangle is untouched
    other = np.tril(np.ones((n, n)), -1) if uplo == 'U' else np.triu(np.ones((n, n)), 1)
    assert np.array_equal(out[other == 1], C[other == 1])


@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NT")
@pytest.mark.parametrize("diag", "NU")
@pytest.mark.parametrize("m,n", [(64, 64), (200, 70), (33, 129), (1, 3), (700, 5), (1030, 128),
                                 (100, 300)])
def test_trsm(engine, side, uplo, trans, diag, m, n):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = _rng(m * 31 + n)
    ka = m if side == 'L' else n
    T = np.asfortranarray(r.standard_normal((ka, ka)) * 0.1 + np.eye(ka) * 2.0)
    B = np.asfortranarray(r.standard_normal((m, n)))
    ref = o._trsm(side, uplo, trans, diag, 0.5, T, B.copy(order='F'))
    Bd = dev_f(B)
    d.trsm_(side, uplo, trans, diag, 0.5, dev_f(T), Bd)
    assert rel_err(host_f(Bd), ref) <= FP64_RTOL


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n", [1, 17, 64, 65, 128, 300, 1024])
def test_potrf(engine, uplo, n):
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(n, n)
    ref, info_ref = o._potrf(uplo, A.copy(order='F'))
    Ad = dev_f(A)
    _, info = d.potrf_(uplo, Ad)
    assert info == info_ref == 0
    out = host_f(Ad)
    tri = np.triu if uplo == 'U' else np.tril
    assert rel_err(tri(out), tri(ref)) <= FP64_RTOL
    # the other triangle is untouched
    other = tri(np.ones((n, n))) == 0
    assert np.array_equal(out[other], A[other])


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("bad", [0, 40, 64, 200])
def test_potrf_not_posdef(uplo, bad):
    import dagger_gb300 as d
    from oracle import tiled as o
    n = 300
    A = o.spd_uniform(n, 11)
    A[bad, bad] = -100.0
    _, info_ref = o._potrf(uplo, A.copy(order='F'))
    _, info = d.potrf_(uplo, dev_f(A))
    assert info == info_ref == bad + 1


def test_potrf_nan_pivot():
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(100, 3)
    A[10, 10] = np.nan
    _, info = d.potrf_('U', dev_f(A))
    assert info == 11


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NT")
def test_trsv_gemv(uplo, trans):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = _rng(9)
    n = 150
    T = np.asfortranarray(r.standard_normal((n, n)) * 0.05 + np.eye(n))
    x = r.standard_normal(n)
    ref = o._trsv(uplo, trans, 'N', T, x.copy())
    xd = dev_f(x)
    d.trsv_(uplo, trans, 'N', dev_f(T), xd)
    assert rel_err(xd.cpu().numpy(), ref) <= FP64_RTOL
    A = np.asfortranarray(r.standard_normal((n, 90)))
    v = r.standard_normal(90 if trans == 'N' else n)
    y = r.standard_normal(n if trans == 'N' else 90)
    ref = o._gemv(trans, -1.0, A, v, 0.5, y.copy())
    yd = dev_f(y)
    d.gemv_(trans, -1.0, dev_f(A), dev_f(v), 0.5, yd)
    assert rel_err(yd.cpu().numpy(), ref) <= FP64_RTOL
