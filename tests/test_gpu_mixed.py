"""Mixed-precision form: the tcgen05 GEMM building block and the refined solve.

The tensor-core GEMM is compared with a plain PyTorch FP64 evaluation of the
same 16-bit products (tolerance 2e-6 relative to sum |a||b|, the FP32
accumulation bound at these K).  The mixed factor-and-solve is checked
against the FP64 oracle: every result reaches the normwise backward error
target (1e-12), and the solution agrees with LAPACK's FP64 solve to within
kappa * 1e-12 (the forward error such a backward error allows).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc(m, n, k, terms, fp16, bn, alpha=-1.0, beta=1.0, seed=0):
    import torch
    import dagger_gb300 as d
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    dt = torch.float16 if fp16 else torch.bfloat16
    Af = torch.randn(m, k, device="cuda", generator=g)   # row i = K values of column i of A
    Bf = torch.randn(n, k, device="cuda", generator=g)
    Ahi, Bhi = Af.to(dt), Bf.to(dt)
    Alo, Blo = (Af - Ahi.float()).to(dt), (Bf - Bhi.float()).to(dt)
    C0 = torch.randn(n, m, device="cuda", generator=g)   # C column-major m x n (ldc = m)
    C = C0.clone()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = d.lib().dg_gemm_tc_tn(m, n, k, terms, int(fp16), Ahi.data_ptr(),
                               Alo.data_ptr() if terms == 3 else None, k, Bhi.data_ptr(),
                               Blo.data_ptr() if terms == 3 else None, k, alpha, beta,
                               C.data_ptr(), m, bn, status.data_ptr(),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == 0, d._lib.last_error()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    a, b = Ahi.double(), Bhi.double()
    prod = a @ b.T
    if terms == 3:
        prod = prod + a @ Blo.double().T + Alo.double() @ b.T
    ref = alpha * prod + beta * C0.double().T
    scale = (a.abs() @ b.abs().T).max().item() + 1e-30
    err = (C.double().T - ref).abs().max().item()
    return err / scale


@pytest.mark.parametrize("fp16", [0, 1], ids=["bf16", "fp16"])
@pytest.mark.parametrize("terms", [1, 3])
@pytest.mark.parametrize("bn", [128, 256])
@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (256, 512, 1024), (200, 300, 136),
                                   (1, 5, 8), (384, 129, 512)])
def test_tc_gemm(fp16, terms, bn, m, n, k):
    assert _tc(m, n, k, terms, fp16, bn) <= 2e-6


def test_tc_gemm_beta_zero():
    assert _tc(256, 256, 256, 1, 0, 128, alpha=0.5, beta=0.0) <= 2e-6


def _spd(n, cond, seed):
    from oracle import tiled as o
    if cond is None:
        return o.spd_uniform(n, seed)
    return o.spd_spectrum(n, cond, seed)


@pytest.mark.parametrize("precision", ["bf16", "bf16x3", "bf16x6", "fp16", "fp16x3", "fp32"])
@pytest.mark.parametrize("n,nb,cond,nrhs", [(512, 128, None, 3), (1000, 128, 1e2, 1),
                                            (1536, 256, 1e4, 5), (2100, 1024, 1e4, 4)])
def test_mixed_solve(precision, n, nb, cond, nrhs):
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    A = _spd(n, cond, 11)
    B = o.rhs_normal(n, nrhs, 5)
    DA = d.DArray.from_array(A, d.Blocks(nb, nb))
    F = d.cholesky_mixed(DA, precision)
    X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12)
    Xh = X.cpu().numpy()
    berr = o.backward_error(A, Xh, B)
    assert rep["converged"] == 1 and berr.max() <= 1e-12, (rep, berr.max())
    Xr = o.lapack_solve(A, B)
    kappa = np.linalg.cond(A, np.inf)
    # forward error allowed by a backward error of 1e-12 (with a factor for n)
    assert np.abs(Xh - Xr).max() / np.abs(Xr).max() <= 10 * kappa * 1e-12
    st = F.stats()
    assert st["info"] == 0 and st["n"] == n
    F.close()


@pytest.mark.parametrize("n,nb,cond,nrhs", [(512, 128, None, 3), (1000, 128, 1e2, 1),
                                            (2100, 1024, 10.0, 4), (4096, 1024, 1e2, 8)])
def test_mixed_solve_fp8(n, nb, cond, nrhs):
    """The FP8 form (E4M3 trailing updates with a power-of-two scale per
    vector) on well-conditioned matrices: GMRES-IR from the coarse factor
    still reaches a backward error of 1e-12."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    A = _spd(n, cond, 13)
    B = o.rhs_normal(n, nrhs, 6)
    F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), "fp8")
    X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12)
    Xh = X.cpu().numpy()
    berr = o.backward_error(A, Xh, B)
    assert rep["converged"] == 1 and berr.max() <= 1e-12, (rep, berr.max())
    Xr = o.lapack_solve(A, B)
    kappa = np.linalg.cond(A, np.inf)
    assert np.abs(Xh - Xr).max() / np.abs(Xr).max() <= 10 * kappa * 1e-12
    F.close()


@pytest.mark.parametrize("precision", ["bf16", "bf16x3"])
@pytest.mark.parametrize("n,nb,cond,nrhs", [(1536, 256, 1e4, 5), (1000, 128, 1e6, 2),
                                            (700, 128, None, 64)])
def test_mixed_solve_emulated_residual(precision, n, nb, cond, nrhs):
    """With the emulated FP64 engine the refinement's residual runs on the
    tensor cores (K = n): the same targets as the FP64-pipe residual."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    A = _spd(n, cond, 13)
    B = o.rhs_normal(n, nrhs, 6)
    old = d.set_f64_engine("emulated")
    try:
        F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), precision)
        X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12, gmres="auto", max_iter=40)
        F.close()
    finally:
        d.set_f64_engine(old)
    Xh = X.cpu().numpy()
    berr = o.backward_error(A, Xh, B)
    assert rep["converged"] == 1 and berr.max() <= 1e-12, (rep, berr.max())
    Xr = o.lapack_solve(A, B)
    kappa = np.linalg.cond(A, np.inf)
    assert np.abs(Xh - Xr).max() / np.abs(Xr).max() <= 10 * kappa * 1e-12


@pytest.mark.parametrize("precision", ["bf16x3", "fp32"])
def test_gmres_ir_ill_conditioned(precision):
    """kappa = 1e8: refinement with GMRES-IR still reaches 1e-12."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 1024, 128
    A = o.spd_spectrum(n, 1e8, 21)
    B = o.rhs_normal(n, 2, 21)
    F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), precision)
    X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12, gmres="auto", max_iter=40)
    berr = o.backward_error(A, X.cpu().numpy(), B)
    assert rep["converged"] == 1 and berr.max() <= 1e-12, (rep, berr.max(), F.stats())


def test_gmres_forced_matches():
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 768, 128
    A = o.spd_spectrum(n, 1e4, 3)
    B = o.rhs_normal(n, 3, 3)
    F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), "bf16")
    X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12, gmres="always")
    assert rep["used_gmres"] == 1 and rep["converged"] == 1
    assert o.backward_error(A, X.cpu().numpy(), B).max() <= 1e-12


def test_fp64_retry_of_a_failed_fp32_pivot():
    """kappa = 1e9 inside one diagonal block: FP32 POTRF breaks down, the FP64
    retry of the block succeeds and the factorization completes unshifted."""
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 128, 128
    A = o.spd_spectrum(n, 1e9, 4)
    F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), "fp32", auto_shift=False)
    st = F.stats()
    assert st["info"] == 0 and st["retries"] >= 1 and st["shift"] == 0.0, st


def test_shift_when_the_low_precision_factor_breaks_down():
    """kappa = 1e8 across several panels: the FP32-accumulated Schur
    complement loses definiteness; the factor of S A S + shift I is used as a
    preconditioner and GMRES-IR still reaches 1e-12 on A x = b."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 1024, 128
    A = o.spd_spectrum(n, 1e8, 21)
    B = o.rhs_normal(n, 2, 21)
    F = d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), "fp32")
    X, rep = F.solve(torch.from_numpy(B).cuda(), tol=1e-12, max_iter=60)
    assert o.backward_error(A, X.cpu().numpy(), B).max() <= 1e-12, (rep, F.stats())


def test_mixed_not_posdef():
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 512, 128
    A = o.spd_uniform(n, 8)
    A[300, 300] = -5.0
    with pytest.raises(d.PosDefException) as e:
        d.cholesky_mixed(d.DArray.from_array(A, d.Blocks(nb, nb)), "bf16x3")
    assert e.value.info > 0
