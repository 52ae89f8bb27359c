"""Tiled Cholesky factor-and-solve on the GPU vs the oracle.

Cases follow the reference's own tests, restated with seeded numpy inputs
(Julia's rand stream cannot be reproduced without Julia):
  test/array/linalg/cholesky.jl   128 x 128, Blocks(32, 32), A*A' + 128 I
  test/array/linalg/solve.jl      ldiv! with DMatrix and DVector right-hand sides
  test/datadeps.jl:946-984        hand-spawned lower tile DAG, 1000 / 100
  test/mpi_cholesky.jl            64 x 64, Blocks(16, 16), errors < 1e-12
plus the CPU benchmark configuration (N = 4096, Blocks(512, 512), 16 RHS),
ragged tilings, both uplo, non-positive-definite inputs, and the
graph / multi-stream / serial issue orders (results must be bit-identical).
Tolerance for the plain FP64 path: 1e-13 relative to the oracle.
"""
import numpy as np
import pytest

from helpers import FP64_RTOL, dev_f, host_f, rel_err

pytestmark = pytest.mark.gpu


def _darray(A, nb):
    import dagger_gb300 as d
    return d.DArray.from_array(A, d.Blocks(nb, nb))


def test_reference_cholesky_recipe():
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(42)
    A = r.random((128, 128))
    A = A @ A.T
    A[np.diag_indices(128)] += 128
    A = np.asfortranarray(A)
    DA = _darray(A, 32)
    assert d.ishermitian(DA) and d.issymmetric(DA)
    C = d.cholesky(DA)
    Uref, _ = o.lapack_factor(A, 'U')
    tol = np.sqrt(np.finfo(float).eps)
    assert rel_err(C.U.cpu().numpy(), Uref) <= tol
    assert rel_err(C.L.cpu().numpy(), Uref.T) <= tol
    # cholesky did not modify DA
    assert np.array_equal(DA.numpy(), A)
    # in place
    C2 = d.cholesky_(DA)
    assert C2.factors is DA
    assert rel_err(np.triu(DA.numpy()), Uref) <= tol
    # random non-symmetric matrix is not hermitian (Blocks(4, 4) on 32 x 32)
    D = _darray(np.asfortranarray(r.random((32, 32))), 4)
    assert not d.ishermitian(D)


def test_ishermitian_tolerance():
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(96, 1)
    B = A.copy(order='F')
    B[70, 3] *= 1 + 1e-12          # off-diagonal pair within sqrt(eps)
    assert d.ishermitian(_darray(B, 32)) == o.ishermitian_tiled(B, 32) == True  # noqa: E712
    B[70, 3] *= 1 + 1e-3           # beyond sqrt(eps)
    assert d.ishermitian(_darray(B, 32)) == o.ishermitian_tiled(B, 32) == False  # noqa: E712
    C = A.copy(order='F')
    C[5, 7] += 1e-15 * C[5, 7]     # inside a diagonal tile: must be exact
    assert d.ishermitian(_darray(C, 32)) == o.ishermitian_tiled(C, 32) == False  # noqa: E712


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb", [(64, 16), (128, 32), (130, 32), (1000, 100), (1024, 128),
                                  (1000, 128), (300, 300), (200, 512)])
def test_factor_vs_oracle(uplo, n, nb):
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(n, n + nb)
    F, info = o.chol_tiled(A, nb, uplo)
    assert info == 0
    C = d.cholesky(_darray(A, nb), uplo)
    G = C.factors.numpy()
    tri = np.triu if uplo == 'U' else np.tril
    assert rel_err(tri(G), tri(F)) <= FP64_RTOL
    # the other triangle keeps the input
    mask = tri(np.ones((n, n))) == 0
    assert np.array_equal(G[mask], A[mask])
    assert o.factor_residual(A, G, uplo) < 1e-14


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb,nrhs", [(128, 32, 128), (128, 64, 7), (1000, 100, 16),
                                       (1000, 128, 1), (513, 128, 200)])
def test_solve_vs_oracle(uplo, n, nb, nrhs):
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(n, 3 * n)
    B = o.rhs_normal(n, nrhs, n)
    F, _ = o.chol_tiled(A, nb, uplo)
    X = B.copy(order='F')
    o.ldiv_cholesky(F, uplo, X, nb)
    C = d.cholesky(_darray(A, nb), uplo)
    DB = _darray(B, nb)
    d.ldiv_(C, DB)
    Xg = DB.numpy()
    assert rel_err(Xg, X) <= FP64_RTOL
    assert o.backward_error(A, Xg, B).max() < 1e-14


@pytest.mark.parametrize("uplo", "UL")
def test_solve_vector_rhs(uplo):
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 300, 64
    A = o.spd_uniform(n, 5)
    b = o.rhs_normal(n, 1, 9)[:, 0].copy()
    F, _ = o.chol_tiled(A, nb, uplo)
    x = b.copy()
    o.ldiv_cholesky(F, uplo, x, nb)
    C = d.cholesky(_darray(A, nb), uplo)
    Db = d.DArray.from_array(b, d.Blocks(nb))
    d.ldiv_(C, Db)
    assert rel_err(Db.numpy(), x) <= 1e-10  # the reference's tolerance (solve.jl:71)
    assert rel_err(Db.numpy(), x) <= FP64_RTOL


def test_reference_solve_recipe():
    """test/array/linalg/solve.jl:46-71: A = A'A + I, N = 128."""
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(7)
    for bs in (64, 128):
        A = r.random((128, 128))
        A = np.asfortranarray(A.T @ A + np.eye(128))
        B = np.asfortranarray(r.random((128, 128)))
        DB = _darray(B, bs)
        d.ldiv_(d.cholesky(_darray(A, bs)), DB)
        ref = o.lapack_solve(A, B)
        assert rel_err(DB.numpy(), ref) <= np.sqrt(np.finfo(float).eps)


def test_mpi_recipe_errors():
    """test/mpi_cholesky.jl: 64 x 64, Blocks(16, 16); both errors < 1e-12."""
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(42)
    A = r.random((64, 64))
    A = A @ A.T
    A[np.diag_indices(64)] += 64
    A = np.asfortranarray(A)
    DA = _darray(A, 16)
    d.cholesky_(DA, 'U')
    U = np.triu(DA.numpy())
    Uref, _ = o.lapack_factor(A, 'U')
    assert np.linalg.norm(U - Uref) / np.linalg.norm(Uref) < 1e-12
    assert np.linalg.norm(U.T @ U - A) / np.linalg.norm(A) < 1e-12


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("bad", [0, 5, 40, 127])
def test_not_posdef(uplo, bad):
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(128, 77)
    A[bad, bad] = -100.0
    _, info_ref = o.chol_tiled(A, 32, uplo)
    with pytest.raises(d.PosDefException) as e:
        d.cholesky(_darray(A, 32), uplo)
    assert e.value.info == info_ref == bad + 1
    C = d.cholesky(_darray(A, 32), uplo, check_=False)
    assert C.info == bad + 1 and not C.issuccess()


def test_issue_orders_bit_identical():
    """Graph, multi-stream and serial issue of the same region give the same bits."""
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 700, 128
    A = o.spd_uniform(n, 99)
    outs = []
    for use_graph, serial in [(True, False), (False, False), (False, True), (True, True)]:
        DA = _darray(A, nb)
        M = DA.chunks
        with d.spawn_datadeps(use_graph=use_graph, serial=serial):
            _spawn_lower_cholesky(d, M, DA.mt)
        outs.append(DA.numpy())
    for x in outs[1:]:
        assert np.array_equal(np.tril(x), np.tril(outs[0]))


def _spawn_lower_cholesky(d, M, mt):
    # the hand-spawned DAG of test/datadeps.jl:960-975
    for k in range(mt):
        d.spawn(d.potrf_, 'L', d.InOut(M[k][k]))
        for m in range(k + 1, mt):
            d.spawn(d.trsm_, 'R', 'L', 'T', 'N', 1.0, d.In(M[k][k]), d.InOut(M[m][k]))
        for n in range(k + 1, mt):
            d.spawn(d.syrk_, 'L', 'N', -1.0, d.In(M[n][k]), 1.0, d.InOut(M[n][n]))
            for m in range(n + 1, mt):
                d.spawn(d.gemm_, 'N', 'T', -1.0, d.In(M[m][k]), d.In(M[n][k]), 1.0,
                        d.InOut(M[m][n]))


def test_reference_datadeps_recipe():
    """test/datadeps.jl:946-984: M = rand*rand' (1000, nb 100) vs LAPACK.potrf!('L')."""
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(3)
    M = r.random((1000, 1000))
    M = np.asfortranarray(M @ M.T)
    expected, info = o._potrf('L', M.copy(order='F'))
    assert info == 0
    DA = _darray(M, 100)
    with d.spawn_datadeps():
        _spawn_lower_cholesky(d, DA.chunks, DA.mt)
    out = DA.numpy()
    assert rel_err(np.tril(out), np.tril(expected)) <= np.sqrt(np.finfo(float).eps)


def test_cpu_config_4096():
    """N = 4096, Blocks(512, 512), A = B B'/N + N I, 16 RHS vs the threaded oracle."""
    import dagger_gb300 as d
    from oracle import native, tiled as o
    n, nb = 4096, 512
    A = o.spd_uniform(n, 2024)
    B = o.rhs_normal(n, 16, 2024)
    native.set_blas_threads(1)
    F, info = native.chol_tiled(A, nb, 'U', nthreads=8)
    assert info == 0
    X = B.copy(order='F')
    native.ldiv_tiled(F, 'U', X, nb, nthreads=8)
    C = d.cholesky(_darray(A, nb), 'U')
    G = C.factors.numpy()
    assert rel_err(np.triu(G), np.triu(F)) <= FP64_RTOL
    DB = _darray(B, nb)
    d.ldiv_(C, DB)
    Xg = DB.numpy()
    assert rel_err(Xg, X) <= FP64_RTOL
    assert o.backward_error(A, Xg, B).max() < 1e-14
