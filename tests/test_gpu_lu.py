"""Tiled LU (src/array/lu.jl) and the solve with it (linalg.jl:264-308) through
libdaggergb300, against the oracle's restatement (oracle/lu.py) and the
committed golden fixtures, on the FP64 pipe and with the emulated FP64
engine.

Tolerances: with the same pivots (the row-by-row partial pivoting of LAPACK,
asserted identical), the factors of two backward-stable orderings of the same
LU differ by rounding amplified by the element growth; 1e-12 of the largest
factor entry (normwise relative) leaves room for that at these sizes, the
reference's own pivoted test asks P*A ≈ L*U to rtol 1e-12 and the oracle
matches untiled LAPACK to 1e-12.  Unpivoted cases run on diagonally dominant
matrices (growth below 2) and are held to the plain path's 1e-13."""
import os

import numpy as np
import pytest

from helpers import FP64_RTOL, dev_f, host_f, rel_err

pytestmark = pytest.mark.gpu

LU_RTOL = 1e-12
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(params=["dfma", "emulated"])
def engine(request):
    import dagger_gb300 as d
    old = d.set_f64_engine(request.param)
    yield request.param
    d.set_f64_engine(old)


def _lapack(A):
    from scipy.linalg import lapack
    lu, piv, info = lapack.dgetrf(np.asfortranarray(A))
    return lu, piv.astype(np.int64) + 1, int(info)


@pytest.mark.parametrize("m,n", [(1, 1), (5, 5), (33, 33), (100, 70), (70, 100), (257, 257),
                                 (1000, 1000), (3000, 200), (64, 1500)])
def test_getrf_matches_lapack(engine, m, n):
    import dagger_gb300 as d
    from oracle import lu as o
    A = o.rand_uniform(m, n, 7 * m + n)
    T = dev_f(A)
    _, ipiv, info = d.getrf_(T)
    F = host_f(T)
    Fl, pl, il = _lapack(A)
    assert info == il == 0
    assert np.array_equal(ipiv.cpu().numpy(), pl)
    assert rel_err(F, Fl) <= LU_RTOL
    assert o.lu_residual(A, F, ipiv.cpu().numpy()) <= LU_RTOL


def test_getrf_zero_pivots_like_lapack():
    import dagger_gb300 as d
    from oracle import lu as o
    A = np.asfortranarray(np.ones((128, 128)))
    T = dev_f(A)
    _, _, info = d.getrf_(T)
    assert info == _lapack(A)[2] == 2
    B = o.rand_uniform(96, 96, 4)
    B[:, 70] = 0.0
    T = dev_f(B)
    _, ipiv, info = d.getrf_(T)
    Fl, pl, il = _lapack(B)
    assert info == il == 71
    assert np.array_equal(ipiv.cpu().numpy(), pl)
    assert rel_err(host_f(T), Fl) <= LU_RTOL


@pytest.mark.parametrize("m,n,nb", [(128, 128, 64), (128, 128, 32), (130, 130, 32),
                                    (300, 200, 64), (200, 300, 64), (1000, 1000, 128),
                                    (1030, 1030, 512), (2048, 2048, 512), (1500, 1500, 1024)])
def test_lu_rowmaximum_matches_oracle(engine, m, n, nb):
    import dagger_gb300 as d
    from oracle import lu as o
    A = o.rand_uniform(m, n, m + 3 * n + nb)
    F0, p0, i0 = o.lu_rowmaximum(A, nb)
    DA = d.DArray.from_array(A, d.Blocks(nb, nb))
    F = d.lu_(DA, "RowMaximum")
    assert F.info == i0 == 0
    assert np.array_equal(F.ipiv.cpu().numpy(), p0)
    got = DA.numpy()
    assert rel_err(got, F0) <= LU_RTOL
    assert o.lu_residual(A, got, p0) <= LU_RTOL


@pytest.mark.parametrize("m,n,nb", [(300, 300, 64), (200, 150, 64), (150, 200, 64), (1024, 1024, 256)])
def test_lu_nopivot_matches_oracle(engine, m, n, nb):
    import dagger_gb300 as d
    from oracle import lu as o
    A = o.rand_uniform(m, n, m + n)
    A[np.diag_indices(min(m, n))] += float(max(m, n))
    F0, p0, i0 = o.lu_nopivot(A, nb)
    DA = d.DArray.from_array(A, d.Blocks(nb, nb))
    F = d.lu_(DA, "NoPivot")
    assert F.info == i0 == 0
    assert np.array_equal(F.ipiv.cpu().numpy(), np.arange(1, min(m, n) + 1))
    assert rel_err(DA.numpy(), F0) <= FP64_RTOL


@pytest.mark.parametrize("nrhs", [0, 1, 5, 64, 300])
def test_lu_solve_matches_oracle(engine, nrhs):
    import dagger_gb300 as d
    from oracle import lu as o
    n, nb = 700, 128
    A = o.rand_uniform(n, n, 31)
    F0, p0, _ = o.lu_rowmaximum(A, nb)
    r = np.random.default_rng(nrhs)
    B = np.asfortranarray(r.standard_normal(n) if nrhs == 0 else r.standard_normal((n, nrhs)))
    X0 = o.ldiv_lu(F0, p0, B.copy(), nb)
    F = d.lu(d.DArray.from_array(A, d.Blocks(nb, nb)))
    part = d.Blocks(nb) if nrhs == 0 else d.Blocks(nb, nb)
    DB = d.DArray.from_array(B, part)
    d.ldiv_(F, DB)
    X = DB.numpy()
    assert rel_err(X, X0) <= 1e-11
    R = B.reshape(n, -1) - A @ X.reshape(n, -1)
    berr = np.abs(R).max(0) / (np.abs(A).sum(1).max() * np.abs(X.reshape(n, -1)).max(0)
                               + np.abs(B.reshape(n, -1)).max(0))
    assert berr.max() <= 1e-14


def test_lu_reference_recipe(engine):
    """test/array/linalg/lu.jl:17-100: rand(128, 128) in Blocks(64, 64), out of
    place (A untouched), P*A ≈ L*U, A \\ b, non-square Blocks(64, 32), and
    SingularException for ones(128, 128)."""
    import torch
    import dagger_gb300 as d
    from oracle import lu as o
    A = o.rand_uniform(128, 128, 1)
    DA = d.DArray.from_array(A, d.Blocks(64, 64))
    F = d.lu(DA, "RowMaximum")
    assert np.array_equal(DA.numpy(), A)
    L, U, P = F.L.cpu().numpy(), F.U.cpu().numpy(), F.P.numpy()
    assert np.linalg.norm(P @ A - L @ U) <= 1e-12 * np.linalg.norm(P @ A)
    assert np.array_equal(U, np.triu(U)) and np.array_equal(L, np.tril(L))
    assert np.allclose(P.T @ P, np.eye(128))
    b = np.random.default_rng(2).random(128)
    x = d.ldiv(F, b).numpy()
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)
    # non-square blocks are re-blocked to Blocks(32, 32)
    A2 = o.rand_uniform(128, 128, 5)
    D2 = d.DArray.from_array(A2, d.Blocks(64, 32))
    F2 = d.lu(D2, "RowMaximum")
    L2, U2, P2 = F2.L.cpu().numpy(), F2.U.cpu().numpy(), F2.P.numpy()
    assert np.linalg.norm(P2 @ A2 - L2 @ U2) <= 1e-12 * np.linalg.norm(A2)
    with pytest.raises(d.SingularException) as e:
        d.lu(d.DArray.from_array(np.ones((128, 128)), d.Blocks(64, 64)))
    assert e.value.info == 2
    G = d.lu(d.DArray.from_array(np.ones((128, 128)), d.Blocks(64, 64)), allowsingular=True)
    assert G.info == 2 and not G.issuccess()
    Z = np.ones((64, 64))
    Z[3, 5] = np.nan
    with pytest.raises(ValueError):
        d.lu(d.DArray.from_array(Z, d.Blocks(32, 32)))
    del torch


@pytest.mark.parametrize("name", ["lu_rowmax_128_64", "lu_rowmax_ragged_200x150_64",
                                  "lu_nopiv_96_32", "lu_solve_160_32_r5"])
def test_lu_golden_fixtures(engine, name):
    import dagger_gb300 as d
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    nb = int(z["nb"])
    A = np.asfortranarray(z["A"])
    if "B" in z:
        F = d.lu(d.DArray.from_array(A, d.Blocks(nb, nb)))
        DB = d.DArray.from_array(np.asfortranarray(z["B"]), d.Blocks(nb, nb))
        d.ldiv_(F, DB)
        assert rel_err(DB.numpy(), z["tiled"]) <= 1e-11
        return
    pivot = "RowMaximum" if str(z["pivot"]) == "rowmaximum" else "NoPivot"
    DA = d.DArray.from_array(A, d.Blocks(nb, nb))
    F = d.lu_(DA, pivot)
    assert np.array_equal(F.ipiv.cpu().numpy(), z["ipiv"])
    assert rel_err(DA.numpy(), z["tiled"]) <= LU_RTOL


def test_lu_large_properties():
    """N = 4096 in Blocks(1024, 1024) with the emulated engine: P A = L U and
    the solve's backward error, checked on the GPU with torch's FP64 matmul
    (size-independent properties; the oracle covers the small sizes)."""
    import torch
    import dagger_gb300 as d
    from oracle import lu as o
    old = d.set_f64_engine("emulated")
    try:
        n, nb = 4096, 1024
        A = o.rand_uniform(n, n, 77)
        DA = d.DArray.from_array(A, d.Blocks(nb, nb))
        F = d.lu(DA)
        Fd = F.factors.collect()
        L = torch.tril(Fd, -1) + torch.eye(n, dtype=torch.float64, device=Fd.device)
        U = torch.triu(Fd)
        At = torch.from_numpy(np.ascontiguousarray(A)).cuda()
        PA = At[F.p.cuda()]
        res = (torch.linalg.norm(PA - L @ U) / torch.linalg.norm(At)).item()
        assert res <= 1e-13
        B = torch.randn(n, 16, dtype=torch.float64, device="cuda", generator=None)
        DB = d.DArray.from_array(B, d.Blocks(nb, nb))
        d.ldiv_(F, DB)
        X = DB.collect()
        R = B - At @ X
        berr = (R.abs().amax(0) / (At.abs().sum(1).amax() * X.abs().amax(0) + B.abs().amax(0))).max().item()
        assert berr <= 1e-14
    finally:
        d.set_f64_engine(old)
