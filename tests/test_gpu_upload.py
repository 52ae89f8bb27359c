"""cholesky_distribute: cholesky(distribute(A, Blocks(nb, nb))) with A on the
host, the tiles uploaded by tasks of the factorization's own graph.

The upload is an exact copy and the factorization's tasks are the same, so the
factor (and, with the emulated engine, the kept inverses) must equal the one
from an eager upload bit for bit; the solve meets the oracle's bar.
"""
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


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("n,nb", [(1000, 128), (2048, 1024), (700, 64), (300, 300)])
def test_upload_factor_matches_eager(engine, uplo, n, nb):
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(n, n + 5)
    A_h = torch.from_numpy(A).pin_memory()
    C1 = d.cholesky_distribute(A_h, d.Blocks(nb, nb), uplo)
    C2 = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), uplo)
    assert torch.equal(C1.factors.collect(), C2.factors.collect())
    if engine == "emulated" and nb <= 1024:
        for k in range((n + nb - 1) // nb):  # the used part of each tile's slot
            r = min(nb, n - k * nb)
            assert torch.equal(C1.winv[k * nb * nb:k * nb * nb + r * r],
                               C2.winv[k * nb * nb:k * nb * nb + r * r])
    else:
        assert C1.winv is None
    F, info = o.chol_tiled(A, nb, uplo)
    tri = np.triu if uplo == 'U' else np.tril
    assert info == 0 and rel_err(tri(C1.factors.numpy()), tri(F)) <= FP64_RTOL


def test_upload_solve_and_reuse(engine):
    """Into a given DArray, repeated (the cached graph), then ldiv_."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb, r = 1500, 512, 16
    out = d.DArray((n, n), d.Blocks(nb, nb))
    B = o.rhs_normal(n, r, 9)
    for seed in (1, 2):
        A = o.spd_uniform(n, 3 * n + seed)
        C = d.cholesky_distribute(A, d.Blocks(nb, nb), 'U', out=out)   # numpy: pinned copy
        assert C.factors is out
        DB = d.DArray.from_array(B, d.Blocks(nb, nb))
        d.ldiv_(C, DB)
        F, _ = o.chol_tiled(A, nb, 'U')
        X = B.copy(order='F')
        o.ldiv_cholesky(F, 'U', X, nb)
        assert rel_err(DB.numpy(), X) <= FP64_RTOL


def test_upload_not_posdef(engine):
    import dagger_gb300 as d
    from oracle import tiled as o
    A = o.spd_uniform(256, 77)
    A[100, 100] = -5.0
    _, info_ref = o.chol_tiled(A, 64, 'U')
    with pytest.raises(d.PosDefException) as e:
        d.cholesky_distribute(A, d.Blocks(64, 64), 'U')
    assert e.value.info == info_ref == 101
    C = d.cholesky_distribute(A, d.Blocks(64, 64), 'U', check_=False)
    assert C.info == 101 and C.winv is None


def test_upload_rejects_pageable_memory():
    """The kernels read the source directly: pageable host memory is refused
    before anything is launched."""
    import torch
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 256, 64
    A = np.ascontiguousarray(o.spd_uniform(n, 3))
    D = d.DArray((n, n), d.Blocks(nb, nb))
    s = torch.cuda.current_stream().cuda_stream
    rc = d.lib().dg_cholesky_tiled_host(b'U', n, nb, A.ctypes.data, n, D.tile_ptrs(), None, s)
    assert rc == -4
    rc = d.lib().dg_cholesky_tiled_host(b'U', n, nb, A.ctypes.data, n - 1, D.tile_ptrs(), None, s)
    assert rc == -5


def test_upload_from_library_host_buffer():
    """A source in dg_host_alloc memory (what a binding without torch uses)."""
    import ctypes
    import dagger_gb300 as d
    from oracle import tiled as o
    n, nb = 640, 128
    L = d.lib()
    A = np.ascontiguousarray(o.spd_uniform(n, 21))
    p = ctypes.c_void_p()
    assert L.dg_host_alloc(A.nbytes, ctypes.byref(p)) == 0
    try:
        H = np.ctypeslib.as_array((ctypes.c_double * (n * n)).from_address(p.value)).reshape(n, n)
        H[:] = A
        D = d.DArray((n, n), d.Blocks(nb, nb))
        import torch
        s = torch.cuda.current_stream().cuda_stream
        assert L.dg_cholesky_tiled_host(b'L', n, nb, p.value, n, D.tile_ptrs(), None, s) == 0
        C = d.cholesky(d.DArray.from_array(A, d.Blocks(nb, nb)), 'L')
        assert torch.equal(D.collect(), C.factors.collect())
    finally:
        assert L.dg_host_free(p) == 0
