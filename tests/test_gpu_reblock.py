"""Re-blocking at the drop-in boundary (maybe_copy_buffered,
src/array/copy.jl:3-37) and the device chkfinite (linalg.jl:126-148).

The reference moves an argument whose Blocks differ from what a region
needs into a buffer of the needed Blocks and copies it back afterwards:
  _chol!    A => Blocks(min_bs, min_bs)                   (cholesky.jl:34)
  ldiv!     factor => Blocks(min_bsa, min_bsa), B => Blocks(min_bsa, ...)
                                                          (linalg.jl:362-404)
  mul!      every operand to the smallest blocking        (mul.jl:11-94)
  ishermitian / lu!  A => Blocks(min, min)                (linalg.jl:96-103)
The copy itself is checked bit for bit; each caller is checked against the
oracle run at the re-blocked tiling (1e-13 normwise) and against the
reference's own recipe (test/array/linalg/solve.jl: N = 128, Blocks(128,
128) and Blocks(64, 128), A'A + I, DMatrix and DVector right-hand sides).
"""
import numpy as np
import pytest

from helpers import FP64_RTOL, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,src,dst", [((130, 70), (32, 32), (64, 16)),
                                           ((128, 128), (128, 128), (64, 64)),
                                           ((100, 1), (7, 1), (64, 1)),
                                           ((1000, 333), (100, 60), (128, 128)),
                                           ((5, 3), (2, 3), (1, 1))])
def test_copy_reblock_bit_exact(shape, src, dst):
    import dagger_gb300 as d
    r = np.random.default_rng(shape[0])
    A = r.standard_normal(shape)
    S = d.DArray.from_array(A, d.Blocks(*src))
    D = d.DArray(shape, d.Blocks(*dst))
    d.copy_reblock(S, D)
    assert np.array_equal(D.numpy(), A)
    back = d.DArray(shape, d.Blocks(*src))
    d.copy_reblock(D, back)
    assert np.array_equal(back.numpy(), A)


def test_copy_reblock_vector():
    import dagger_gb300 as d
    b = np.random.default_rng(3).standard_normal(257)
    S = d.DArray.from_array(b, d.Blocks(100))
    D = d.DArray((257,), d.Blocks(64))
    d.copy_reblock(S, D)
    assert np.array_equal(D.numpy(), b)


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("engine", ["dfma", "emulated"])
def test_cholesky_nonsquare_blocks(uplo, engine):
    """_chol! on Blocks(64, 32): factored at Blocks(32, 32) and copied back;
    the result keeps the caller's Blocks."""
    import dagger_gb300 as d
    from oracle import tiled as o
    old = d.set_f64_engine(engine)
    try:
        A = o.spd_uniform(200, 9)
        F, info = o.chol_tiled(A, 32, uplo)
        assert info == 0
        DA = d.DArray.from_array(A, d.Blocks(64, 32))
        C = d.cholesky(DA, uplo)
        assert C.factors.partitioning == d.Blocks(64, 32)
        tri = np.triu if uplo == 'U' else np.tril
        G = C.factors.numpy()
        assert rel_err(tri(G), tri(F)) <= FP64_RTOL
        assert np.array_equal(DA.numpy(), A)      # cholesky copies (cholcopy)
        assert d.ishermitian(DA)
    finally:
        d.set_f64_engine(old)


@pytest.mark.parametrize("engine", ["dfma", "emulated"])
@pytest.mark.parametrize("bs_i", [128, 64])
def test_reference_solve_recipe(engine, bs_i):
    """test/array/linalg/solve.jl:46-71 with Blocks(bs_i, 128): cholesky(DA)
    then ldiv! with a DMatrix and a DVector right-hand side ≈ LAPACK."""
    import dagger_gb300 as d
    import scipy.linalg as sl
    from oracle import tiled as o
    old = d.set_f64_engine(engine)
    try:
        r = np.random.default_rng(bs_i)
        N = 128
        A = r.random((N, N))
        A = A.T @ A + np.eye(N)
        B = r.random((N, N))
        DA = d.DArray.from_array(A, d.Blocks(bs_i, 128))
        DB = d.DArray.from_array(B, d.Blocks(bs_i, 128))
        C = d.cholesky(DA)
        d.ldiv_(C, DB)
        X = sl.cho_solve(sl.cho_factor(A), B)
        assert np.allclose(DB.numpy(), X, rtol=np.sqrt(np.finfo(float).eps))
        assert DB.partitioning == d.Blocks(bs_i, 128)
        # the oracle at the re-blocked tiling: Blocks(min_bsa, min_bsa)
        mb = min(bs_i, 128)
        F, _ = o.chol_tiled(A, mb, 'U')
        Xo = np.asfortranarray(B.copy())
        o.ldiv_cholesky(F, 'U', Xo, mb)
        assert rel_err(DB.numpy(), Xo) <= FP64_RTOL
        b = r.random(N)
        Db = d.DArray.from_array(b, d.Blocks(bs_i))
        d.ldiv_(d.cholesky(DA), Db)
        xb = sl.cho_solve(sl.cho_factor(A), b)
        assert np.allclose(Db.numpy(), xb, rtol=1e-10)
    finally:
        d.set_f64_engine(old)


@pytest.mark.parametrize("uplo", "UL")
def test_ldiv_rhs_blocked_differently(uplo):
    """A Blocks(128, 128) factor and B in Blocks(64, 64): B is solved at
    Blocks(128, 128) and copied back into its own blocking."""
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(300, 4)
    B = o.rhs_normal(300, 70, 4)
    C = d.cholesky(d.DArray.from_array(A, d.Blocks(128, 128)), uplo)
    DB = d.DArray.from_array(B, d.Blocks(64, 64))
    d.ldiv_(C, DB)
    F, _ = o.chol_tiled(A, 128, uplo)
    X = np.asfortranarray(B.copy())
    o.ldiv_cholesky(F, uplo, X, 128)
    assert DB.partitioning == d.Blocks(64, 64)
    assert rel_err(DB.numpy(), X) <= FP64_RTOL


def test_mul_mixed_blocks():
    """mul! with operands in different Blocks: the products run at the
    smallest block size and C keeps its own Blocks."""
    import dagger_gb300 as d
    r = np.random.default_rng(8)
    A = r.standard_normal((200, 150))
    B = r.standard_normal((150, 90))
    C0 = r.standard_normal((200, 90))
    DA = d.DArray.from_array(A, d.Blocks(64, 64))
    DB = d.DArray.from_array(B, d.Blocks(32, 32))
    DC = d.DArray.from_array(C0, d.Blocks(50, 40))
    d.mul_(DC, DA, DB, 2.0, -1.0)
    assert DC.partitioning == d.Blocks(50, 40)
    assert rel_err(DC.numpy(), 2.0 * A @ B - C0) <= FP64_RTOL
    S = d.DArray((200, 200), d.Blocks(64, 64))
    DG = d.DArray.from_array(A, d.Blocks(40, 30))
    d.mul_(S, DG, DG, 1.0, 0.0, 'N', 'T')        # A === B: syrk_dagger!
    assert rel_err(S.numpy(), A @ A.T) <= FP64_RTOL


def test_ishermitian_nonsquare_blocks():
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(96, 2)
    assert d.ishermitian(d.DArray.from_array(A, d.Blocks(32, 16)))
    A[5, 70] += 1.0
    assert not d.ishermitian(d.DArray.from_array(A, d.Blocks(32, 16)))


@pytest.mark.parametrize("where", ["none", "random", "diagonal", "ragged", "first", "last"])
@pytest.mark.parametrize("bad", [np.inf, -np.inf, np.nan])
def test_chkfinite_on_device(where, bad):
    """LAPACK.chkfinite(::DArray) (linalg.jl:126-148) on 300 x 300 with
    Blocks(64, 64): the last row and column of tiles are ragged (44)."""
    import dagger_gb300 as d
    r = np.random.default_rng(1)
    A = r.standard_normal((300, 300))
    pos = {"none": None, "random": (100, 170), "diagonal": (130, 140), "ragged": (299, 257),
           "first": (0, 0), "last": (299, 299)}[where]
    if pos is not None:
        A[pos] = bad
    expect = bool(np.isfinite(A).all())
    DA = d.DArray.from_array(A, d.Blocks(64, 64))
    if expect:
        assert d.chkfinite(DA) is True
        assert d.lib().dg_chkfinite_tiled(300, 64, DA.tile_ptrs(), None) == 1
    else:
        with pytest.raises(ValueError):
            d.chkfinite(DA)
        assert d.lib().dg_chkfinite_tiled(300, 64, DA.tile_ptrs(), None) == 0


@pytest.mark.parametrize("shape,part", [((200, 77), (64, 32)), ((33, 500), (8, 128)),
                                        ((1, 1), (1, 1)), ((129,), (64,))])
def test_chkfinite_rectangular(shape, part):
    import dagger_gb300 as d
    r = np.random.default_rng(2)
    A = r.standard_normal(shape)
    DA = d.DArray.from_array(A, d.Blocks(*part))
    assert d.chkfinite(DA)
    A.flat[A.size - 1] = np.nan
    with pytest.raises(ValueError):
        d.chkfinite(d.DArray.from_array(A, d.Blocks(*part)))
