"""FP64 engine 2: the trailing SYRK/GEMM tile updates emulated on the BF16
tensor cores (7 slices of 8 bits per vector, exact products, FP64 sum).

The building block is checked against numpy's FP64 GEMM with the bound of an
FP64 GEMM taken over each output's vectors:
    |C - C_ref|_ij <= 4e-16 * k * max_p |A(p, i)| * max_p |B(p, j)| * |alpha|
                      + 2^-51 (|beta C0|_ij + |C_ref|_ij)
and the tiled Cholesky run with engine 2 is held to the plain path's parity
bar against the oracle (1e-13 normwise, both uplo, ragged tilings, tile
sizes that are not multiples of 8), with the oracle's LAPACK info on
non-positive-definite inputs.
"""
import numpy as np
import pytest

from helpers import FP64_RTOL, dev_f, host_f, rel_err

pytestmark = pytest.mark.gpu

GEMM_BOUND = 4e-16


@pytest.fixture
def emulated():
    import dagger_gb300 as d
    old = d.set_f64_engine("emulated")
    yield d
    d.set_f64_engine(old)


def _emulated_gemm_error(m, n, k, alpha, beta, seed, scale_rows=False):
    import dagger_gb300 as d
    r = np.random.default_rng(seed)
    A = np.asfortranarray(r.uniform(-1, 1, (k, m)))
    B = np.asfortranarray(r.standard_normal((k, n)))
    if scale_rows:  # vectors of very different magnitudes
        A *= np.exp2(r.integers(-30, 30, m))[None, :]
        B *= np.exp2(r.integers(-30, 30, n))[None, :]
    C0 = np.asfortranarray(r.standard_normal((m, n)))
    Cg = dev_f(C0)
    d.gemm_f64_emulated_tn(alpha, dev_f(A), dev_f(B), beta, Cg)
    got = host_f(Cg)
    ref = alpha * (A.T @ B) + beta * C0
    # the GEMM bound, plus the roundings of the beta term and of the sum (the
    # kernel fuses them into one FMA, numpy rounds twice)
    bound = GEMM_BOUND * abs(alpha) * k * np.abs(A).max(0)[:, None] * np.abs(B).max(0)[None, :]
    bound = bound + 2.0 ** -51 * (np.abs(beta * C0) + np.abs(ref))
    return float((np.abs(got - ref) / bound).max())


@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (1, 1, 1), (257, 129, 100), (1000, 700, 1024),
                                   (130, 70, 513), (64, 300, 8), (1024, 1024, 1024),
                                   (256, 64, 4096), (300, 100, 33000),
                                   # several output blocks per CTA (one wave over the SMs)
                                   (4096, 1024, 256), (3000, 2000, 100), (2500, 700, 1500)])
def test_emulated_gemm_vs_fp64(m, n, k):
    assert _emulated_gemm_error(m, n, k, -1.0, 1.0, m + n + k) <= 1.0


def test_emulated_gemm_alpha_beta_and_scales():
    assert _emulated_gemm_error(300, 200, 777, 0.37, -2.5, 5, scale_rows=True) <= 1.0
    assert _emulated_gemm_error(200, 300, 256, 2.0, 0.0, 6) <= 1.0


def test_emulated_gemm_exact_on_small_integers():
    """Integers below 2^7 are one slice: the product must be exact."""
    import dagger_gb300 as d
    r = np.random.default_rng(3)
    A = np.asfortranarray(r.integers(-127, 128, (512, 96)).astype(np.float64))
    B = np.asfortranarray(r.integers(-127, 128, (512, 80)).astype(np.float64))
    Cg = dev_f(np.zeros((96, 80), order='F'))
    d.gemm_f64_emulated_tn(1.0, dev_f(A), dev_f(B), 0.0, Cg)
    assert np.array_equal(host_f(Cg), A.T @ B)


def test_emulated_gemm_zero_vectors():
    import dagger_gb300 as d
    r = np.random.default_rng(4)
    A = np.asfortranarray(r.standard_normal((64, 130)))
    A[:, 7] = 0.0
    B = np.asfortranarray(r.standard_normal((64, 70)))
    B[:, 3] = 0.0
    Cg = dev_f(np.ones((130, 70), order='F'))
    d.gemm_f64_emulated_tn(1.0, dev_f(A), dev_f(B), 1.0, Cg)
    got = host_f(Cg)
    assert np.array_equal(got[7, :], np.ones(70))
    assert np.array_equal(got[:, 3], np.ones(130))
    assert rel_err(got, A.T @ B + 1.0) <= 1e-14


def test_emulated_gemm_argument_errors():
    import dagger_gb300 as d
    r = np.random.default_rng(5)
    A = dev_f(r.standard_normal((131073, 2)))
    B = dev_f(r.standard_normal((131073, 2)))
    C = dev_f(np.zeros((2, 2), order='F'))
    with pytest.raises(ValueError):
        d.gemm_f64_emulated_tn(1.0, A, B, 0.0, C)   # k > 131072


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb", [(64, 16), (128, 32), (130, 32), (1000, 100), (1024, 128),
                                  (1000, 128), (300, 300), (2048, 1024), (700, 60)])
def test_factor_engine2_vs_oracle(emulated, uplo, n, nb):
    d = emulated
    from oracle import tiled as o
    A = o.spd_uniform(n, n + nb)
    F, info = o.chol_tiled(A, nb, uplo)
    assert info == 0
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), uplo)
    G = C.factors.numpy()
    tri = np.triu if uplo == 'U' else np.tril
    assert rel_err(tri(G), tri(F)) <= FP64_RTOL
    mask = tri(np.ones((n, n))) == 0
    assert np.array_equal(G[mask], A[mask])
    assert o.factor_residual(A, G, uplo) < 1e-14


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb,nrhs", [(1000, 128, 16), (1500, 512, 64), (900, 300, 1),
                                       (700, 100, 250), (2048, 1024, 130)])
def test_solve_engine2_vs_oracle(emulated, uplo, n, nb, nrhs):
    d = emulated
    from oracle import tiled as o
    A = o.spd_uniform(n, 3 * n)
    B = o.rhs_normal(n, nrhs, n)
    F, _ = o.chol_tiled(A, nb, uplo)
    X = B.copy(order='F')
    o.ldiv_cholesky(F, uplo, X, nb)
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), uplo)
    DB = d.DArray.from_array(B, d.Blocks(nb, nb))
    d.ldiv_(C, DB)
    assert rel_err(DB.numpy(), X) <= FP64_RTOL
    assert o.backward_error(A, DB.numpy(), B).max() < 1e-14


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("bad", [0, 40, 127])
def test_not_posdef_engine2(emulated, uplo, bad):
    d = emulated
    from oracle import tiled as o
    A = o.spd_uniform(128, 77)
    A[bad, bad] = -100.0
    _, info_ref = o.chol_tiled(A, 32, uplo)
    with pytest.raises(d.PosDefException) as e:
        d.cholesky(d.DArray.from_array(A, d.Blocks(32, 32)), uplo)
    assert e.value.info == info_ref == bad + 1


def test_engine2_cpu_config_4096(emulated):
    """N = 4096, Blocks(512, 512), 16 RHS against the threaded oracle."""
    d = emulated
    from oracle import native, tiled as o
    n, nb = 4096, 512
    A = o.spd_uniform(n, 2024)
    B = o.rhs_normal(n, 16, 2024)
    native.set_blas_threads(1)
    F, info = native.chol_tiled(A, nb, 'U', nthreads=8)
    assert info == 0
    X = B.copy(order='F')
    native.ldiv_tiled(F, 'U', X, nb, nthreads=8)
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), 'U')
    assert rel_err(np.triu(C.factors.numpy()), np.triu(F)) <= FP64_RTOL
    DB = d.DArray.from_array(B, d.Blocks(nb, nb))
    d.ldiv_(C, DB)
    assert rel_err(DB.numpy(), X) <= FP64_RTOL


def test_slice_stages_match_one_call():
    """dg_f64_slices + dg_gemm_f64_slices give the bits of the one-call form."""
    import torch
    import dagger_gb300 as d
    L = d.lib()
    r = np.random.default_rng(8)
    k, m, n = 300, 200, 150
    ldk = (k + 7) // 8 * 8
    A = np.asfortranarray(r.standard_normal((k, m)))
    B = np.asfortranarray(r.standard_normal((k, n)))
    C0 = np.asfortranarray(r.standard_normal((m, n)))
    Ad, Bd = dev_f(A), dev_f(B)
    C1 = dev_f(C0)
    d.gemm_f64_emulated_tn(-1.0, Ad, Bd, 1.0, C1)
    sa = torch.empty(7 * ldk * m, dtype=torch.bfloat16, device="cuda")
    sb = torch.empty(7 * ldk * n, dtype=torch.bfloat16, device="cuda")
    ea = torch.empty(m, dtype=torch.int64, device="cuda")
    eb = torch.empty(n, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert L.dg_f64_slices(k, m, Ad.data_ptr(), k, 1, sa.data_ptr(), ldk, ea.data_ptr(), s) == 0
    assert L.dg_f64_slices(k, n, Bd.data_ptr(), k, 1, sb.data_ptr(), ldk, eb.data_ptr(), s) == 0
    C2 = dev_f(C0)
    assert L.dg_gemm_f64_slices(m, n, k, -1.0, sa.data_ptr(), ldk, ea.data_ptr(), sb.data_ptr(),
                                ldk, eb.data_ptr(), 1.0, C2.data_ptr(), m, None, s) == 0
    torch.cuda.synchronize()
    assert np.array_equal(host_f(C1), host_f(C2))


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb,nrhs", [(1000, 128, 16), (2048, 1024, 64), (700, 100, 250)])
def test_solve_engine2_inverse_and_substitution_agree(emulated, uplo, n, nb, nrhs):
    """The solve with the kept inverses and the one by substitution (a
    Cholesky built from the factor alone) both meet the oracle's bar."""
    d = emulated
    from oracle import tiled as o
    A = o.spd_uniform(n, 3 * n + 1)
    B = o.rhs_normal(n, nrhs, n + 1)
    F, _ = o.chol_tiled(A, nb, uplo)
    X = B.copy(order='F')
    o.ldiv_cholesky(F, uplo, X, nb)
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), uplo)
    assert C.winv is not None
    for chol in (C, d.Cholesky(C.factors, uplo, 0)):
        DB = d.DArray.from_array(B, d.Blocks(nb, nb))
        d.ldiv_(chol, DB)
        assert rel_err(DB.numpy(), X) <= FP64_RTOL
        assert o.backward_error(A, DB.numpy(), B).max() < 1e-14


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb", [(1000, 128), (1800, 1024), (2048, 512)])
def test_factor_keeps_diagonal_inverses(emulated, uplo, n, nb):
    """winv holds W_k = U_kk^-T (L_kk^-T) of every diagonal tile, the ragged
    last one included, column-major with ld = the tile's rows (tiles of 256
    rows or more are inverted by halves, the off-diagonal block emulated)."""
    d = emulated
    import torch
    from oracle import tiled as o
    A = o.spd_uniform(n, 11)
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), uplo)
    G = C.factors.numpy()
    W = C.winv.cpu().numpy()
    mt = (n + nb - 1) // nb
    for k in range(mt):
        r = min(nb, n - k * nb)
        T = G[k * nb:k * nb + r, k * nb:k * nb + r]
        T = np.triu(T) if uplo == 'U' else np.tril(T)
        Wk = W[k * nb * nb:k * nb * nb + r * r].reshape(r, r, order='F')
        ref = np.linalg.inv(T).T
        assert np.abs(Wk - ref).max() <= 1e-13 * np.abs(ref).max()


def test_winv_calls_need_the_emulated_engine():
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    L = d.lib()
    old = d.set_f64_engine("dfma")
    try:
        A = d.DArray.from_array(o.spd_uniform(256, 3), d.Blocks(64, 64))
        w = torch.empty(4 * 64 * 64, dtype=torch.float64, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        assert L.dg_cholesky_tiled_winv(b'U', 256, 64, A.tile_ptrs(), w.data_ptr(), s) == -1003
        C = d.cholesky(A, 'U')
        assert C.winv is None
    finally:
        d.set_f64_engine(old)
