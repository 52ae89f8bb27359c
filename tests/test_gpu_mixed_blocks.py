"""Building blocks of the mixed form's critical path.

dg_potrf_inv_f32: the cooperative FP32 factor + inverse of a diagonal block
(n <= 1024, any leading dimension, ragged sizes) against FP64 LAPACK on the
same FP32 input: |U - U_ref| <= 1e-5 |U_ref| (FP32 rounding times the
growth of a well-conditioned block), V U = I to 1e-5, the strict lower parts
untouched (U) and zero (V), and LAPACK's info on a non-positive pivot.

dg_gemm_f32_tc_tn: the FP32-accurate tensor-core GEMM (three BF16 slices per
operand, six products) against an FP64 evaluation: |C - C_ref| <= 4e-6
sum |a||b|, the bound of the tensor cores' FP32 accumulation at these K (the
dropped slice products are below 2^-24 of each product).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def _spd32(n, seed):
    r = np.random.default_rng(seed)
    B = r.uniform(-1, 1, (n, n))
    return (B @ B.T / n + np.eye(n)).astype(np.float32)


@pytest.mark.parametrize("n,ld", [(1, 1), (7, 8), (32, 32), (33, 40), (64, 64), (100, 128),
                                  (250, 256), (512, 512), (777, 1024), (1000, 1000),
                                  (1024, 1024)])
def test_potrf_inv_f32(n, ld):
    import torch
    import dagger_gb300 as d
    A = _spd32(n, n)
    lower_marker = np.float32(7.0)
    M = np.full((ld, n), lower_marker, dtype=np.float32)      # column-major ld x n storage
    iu = np.triu_indices(n)
    M[iu] = A[iu]
    Mt = torch.from_numpy(np.ascontiguousarray(M.T)).cuda()   # (n, ld): column j contiguous
    V = torch.full((n, ld), 5.0, dtype=torch.float32, device="cuda")
    import ctypes
    info = ctypes.c_int(-1)
    rc = d.lib().dg_potrf_inv_f32(n, Mt.data_ptr(), ld, V.data_ptr(), ld, ctypes.byref(info),
                                  _stream())
    assert rc == 0 and info.value == 0, (rc, d._lib.last_error())
    G = Mt.cpu().numpy().T[:n, :n].astype(np.float64)
    Vh = V.cpu().numpy().T[:n, :n].astype(np.float64)
    Uref = np.linalg.cholesky(A.astype(np.float64)).T
    assert np.abs(np.triu(G) - Uref).max() <= 1e-5 * np.abs(Uref).max()
    # the strict lower part of the block is not touched
    assert np.all(G[np.tril_indices(n, -1)] == lower_marker)
    assert np.all(Vh[np.tril_indices(n, -1)] == 0.0)
    assert np.abs(Vh @ np.triu(G) - np.eye(n)).max() <= 1e-5
    # rows past n of a padded column are not written
    if ld > n:
        assert np.all(V.cpu().numpy()[:, n:] == 5.0)


@pytest.mark.parametrize("n,bad", [(64, 0), (100, 37), (1024, 999), (300, 299)])
def test_potrf_inv_f32_not_posdef(n, bad):
    import ctypes
    import torch
    import dagger_gb300 as d
    A = np.eye(n, dtype=np.float32)
    A[bad, bad] = -1.0
    Mt = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    V = torch.zeros(n, n, dtype=torch.float32, device="cuda")
    info = ctypes.c_int(-1)
    rc = d.lib().dg_potrf_inv_f32(n, Mt.data_ptr(), n, V.data_ptr(), n, ctypes.byref(info),
                                  _stream())
    assert rc == bad + 1 and info.value == bad + 1


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (1000, 700, 1024), (1024, 4000, 1024),
                                   (5, 3, 8), (300, 129, 136)])
def test_gemm_f32_tc(m, n, k):
    import torch
    import dagger_gb300 as d
    g = torch.Generator(device="cuda")
    g.manual_seed(m + n + k)
    A = torch.randn(m, k, device="cuda", generator=g)   # column-major k x m: row i of A = column
    B = torch.randn(n, k, device="cuda", generator=g)
    A[:, : k // 2] *= 1e3                              # mixed magnitudes along K
    C0 = torch.randn(n, m, device="cuda", generator=g)  # column-major m x n
    C = C0.clone()
    rc = d.lib().dg_gemm_f32_tc_tn(m, n, k, -0.5, A.data_ptr(), k, B.data_ptr(), k, 2.0,
                                   C.data_ptr(), m, _stream())
    assert rc == 0, d._lib.last_error()
    torch.cuda.synchronize()
    a, b = A.double(), B.double()
    ref = -0.5 * (a @ b.T) + 2.0 * C0.double().T
    bound = 4e-6 * 0.5 * (a.abs() @ b.abs().T) + 2e-7 * (2.0 * C0.double().T).abs() + 1e-30
    assert ((C.double().T - ref).abs() / bound).max().item() <= 1.0


@pytest.mark.parametrize("m,n,k", [(128, 128, 128), (1000, 700, 1024), (1024, 4000, 1024),
                                   (5, 3, 16), (300, 129, 136)])
def test_gemm_f8_tc(m, n, k):
    """E4M3 operands with a power-of-two scale per vector, one kind::f8f6f4
    product, scales applied to the FP32 accumulators: each operand value is
    rounded to 4 significant bits (relative error <= 2^-4), values below
    E4M3's normal range (2^-6 after scaling the vector's largest magnitude
    into [128, 256)) to an absolute 2^-10 of the scaled range."""
    import torch
    import dagger_gb300 as d
    g = torch.Generator(device="cuda")
    g.manual_seed(m + 2 * n + k)
    A = torch.randn(m, k, device="cuda", generator=g)   # column-major k x m
    B = torch.randn(n, k, device="cuda", generator=g)
    A[:, : k // 2] *= 1e3                              # mixed magnitudes along K
    B[: n // 2] *= 1e-20                               # vectors far from 1 in scale
    C0 = torch.randn(n, m, device="cuda", generator=g)
    C = C0.clone()
    rc = d.lib().dg_gemm_f8_tc_tn(m, n, k, -0.5, A.data_ptr(), k, B.data_ptr(), k, 2.0,
                                  C.data_ptr(), m, _stream())
    assert rc == 0, d._lib.last_error()
    torch.cuda.synchronize()
    a, b = A.double(), B.double()
    ref = -0.5 * (a @ b.T) + 2.0 * C0.double().T
    amax = a.abs().amax(dim=1, keepdim=True)            # m x 1
    bmax = b.abs().amax(dim=1, keepdim=True).T          # 1 x n
    sub = 2.0 ** -15 * (amax * b.abs().sum(dim=1, keepdim=True).T
                        + a.abs().sum(dim=1, keepdim=True) * bmax)
    bound = 0.5 * (0.1329 * (a.abs() @ b.abs().T) + sub) + 2e-7 * (2.0 * C0.double().T).abs()
    err = (C.double().T - ref).abs()
    assert (err <= bound + 1e-30).all().item(), (err / (bound + 1e-30)).max().item()
    # the rounding errors are not systematic: the typical error is far below the bound
    rel = (err / (0.5 * (a.abs() @ b.abs().T) + 1e-300)).median().item()
    assert rel <= 2e-2, rel


def test_gemm_f8_tc_nonfinite():
    """A vector holding an infinity or a NaN makes every product with it NaN."""
    import torch
    import dagger_gb300 as d
    m, n, k = 256, 128, 64
    A = torch.randn(m, k, device="cuda")
    B = torch.randn(n, k, device="cuda")
    A[7, 3] = float("inf")
    B[5, 0] = float("nan")
    C = torch.zeros(n, m, device="cuda")
    rc = d.lib().dg_gemm_f8_tc_tn(m, n, k, 1.0, A.data_ptr(), k, B.data_ptr(), k, 0.0,
                                  C.data_ptr(), m, _stream())
    assert rc == 0
    torch.cuda.synchronize()
    Ct = C.T
    assert torch.isnan(Ct[7]).all().item() and torch.isnan(Ct[:, 5]).all().item()
    mask = torch.ones(m, n, dtype=torch.bool, device="cuda")
    mask[7] = False
    mask[:, 5] = False
    assert torch.isfinite(Ct[mask]).all().item()
