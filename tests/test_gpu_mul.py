"""mul! on DArrays (src/array/mul.jl): gemm_dagger! and syrk_dagger! +
copytri! as library graphs, against the oracle's tile loops, on the FP64 pipe
and with the emulated FP64 engine."""
import numpy as np
import pytest

from helpers import FP64_RTOL, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["dfma", "emulated"])
def engine(request):
    import dagger_gb300 as d
    old = d.set_f64_engine(request.param)
    yield request.param
    d.set_f64_engine(old)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,nb", [(700, 300, 500, 128), (256, 256, 256, 64), (1030, 1030, 1024, 512)])
def test_gemm_dagger(engine, ta, tb, m, n, k, nb):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(m + 3 * n + 7 * k)
    A = r.standard_normal((m, k) if ta == "N" else (k, m))
    B = r.standard_normal((k, n) if tb == "N" else (n, k))
    C0 = r.standard_normal((m, n))
    ref = o.gemm_dagger(C0, ta, tb, A, B, -0.75, 1.25, nb)
    P = d.Blocks(nb, nb)
    C = d.DArray.from_array(C0, P)
    d.gemm_dagger_(C, ta, tb, d.DArray.from_array(A, P), d.DArray.from_array(B, P), -0.75, 1.25)
    assert rel_err(C.numpy(), ref) <= FP64_RTOL


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,k,nb", [(700, 500, 128), (1024, 2048, 512), (300, 64, 64)])
def test_syrk_dagger(engine, trans, n, k, nb):
    import dagger_gb300 as d
    from oracle import tiled as o
    r = np.random.default_rng(n + k)
    A = r.standard_normal((n, k) if trans == "N" else (k, n))
    S = r.standard_normal((n, n))
    C0 = S + S.T
    ref = o.syrk_dagger(C0, trans, A, 1.5, -0.5, nb)
    P = d.Blocks(nb, nb)
    C = d.DArray.from_array(C0, P)
    d.syrk_dagger_(C, trans, d.DArray.from_array(A, P), 1.5, -0.5)
    got = C.numpy()
    assert rel_err(got, ref) <= FP64_RTOL
    assert np.array_equal(got, got.T)


def test_mul_dispatch_and_matmul(engine):
    """A' * A takes syrk_dagger! (exactly symmetric); A * B gemm_dagger!;
    beta = 0 ignores C's old contents (NaN there must not leak)."""
    import torch
    import dagger_gb300 as d
    r = np.random.default_rng(11)
    nb = 128
    A = r.standard_normal((600, 400))
    B = r.standard_normal((400, 500))
    P = d.Blocks(nb, nb)
    DA = d.DArray.from_array(A, P)
    G = d.matmul(DA, DA, 'T', 'N')
    g = G.numpy()
    assert np.array_equal(g, g.T) and rel_err(g, A.T @ A) <= FP64_RTOL
    C = d.DArray.from_array(np.full((600, 500), np.nan), P)
    d.mul_(C, DA, d.DArray.from_array(B, P))
    assert rel_err(C.numpy(), A @ B) <= FP64_RTOL


def test_spd_input_then_cholesky(engine):
    """The reference benchmark's input, G*G' (+ n I), built and factored on the
    device (benchmark/suites/linalg.jl:15)."""
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 1024, 256
    r = np.random.default_rng(5)
    G = r.uniform(-1, 1, (n, n))
    P = d.Blocks(nb, nb)
    C = d.DArray.from_array(n * np.eye(n), P)
    d.syrk_dagger_(C, 'N', d.DArray.from_array(G, P), 1.0 / n, 1.0)
    A = C.numpy()
    assert rel_err(A, G @ G.T / n + n * np.eye(n)) <= FP64_RTOL
    F = d.cholesky(C, 'U').factors.numpy()
    assert o.factor_residual(A, F, 'U') < 1e-14


def test_gemm_argument_errors():
    import dagger_gb300 as d
    P = d.Blocks(64, 64)
    A = d.DArray.zeros(P, (128, 64))
    C = d.DArray.zeros(P, (128, 64))
    with pytest.raises(ValueError):
        d.gemm_dagger_(C, 'N', 'N', A, d.DArray.zeros(P, (32, 64)))  # 128x64 times 32x64
    with pytest.raises(ValueError):
        d.gemm_dagger_(C, 'T', 'N', A, d.DArray.zeros(P, (64, 64)))  # 64x128 times 64x64
    assert d.lib().dg_gemm_tiled(b'X', b'N', 1, 1, 1, 1, 1.0, None, None, 0.0, None, None) == -1
