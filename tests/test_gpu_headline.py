"""Parity on the benchmark's own matrix class: N = 16384, Blocks(1024, 1024),
A = Q diag(logspace(0, 4)) Q' (kappa = 1e4, Q from the QR of a seeded
Gaussian, the construction bench.py times at N = 32768), 64 right-hand sides
N(0, 1), both uplo, with the emulated FP64 engine (the benchmark's) and the
plain FP64 pipe, against the oracle's threaded C restatement of _chol! and
ldiv! (src/array/cholesky.jl:19-108, src/array/linalg.jl:352-405) on the
same inputs.

Tolerances (max-norm relative, as every parity test here):
  factor   1e-13: the plain-form gate; two FP64 factorizations of this
           matrix differ by about 1e-14 (measured: LAPACK dpotrf against the
           oracle, N = 4096 and 8192, 3.7e-15 and 3.3e-15).
  solve    1e-12: the solution's sensitivity is kappa times larger; LAPACK
           dpotrs against the oracle already differ by 2.8e-13 and 2.6e-13
           (N = 4096, 8192).  The solve is also held to the oracle's own
           normwise backward error (within 4x).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, NB, NRHS, COND, SEED = 16384, 1024, 64, 1e4, 2024
FACTOR_TOL = 1e-13
SOLVE_TOL = 1e-12


@pytest.fixture(scope="module")
def system():
    import torch
    import bench
    dev = torch.device("cuda", 0)
    A = bench.make_spd_spectrum_gpu(N, COND, SEED, dev)
    B = bench.make_rhs_gpu(N, NRHS, SEED, dev)
    torch.cuda.synchronize()
    An = np.asfortranarray(A.cpu().numpy())   # symmetric: row- and column-major agree
    Bn = np.asfortranarray(B.cpu().numpy())
    yield A, B, An, Bn
    del A, B
    torch.cuda.empty_cache()


_oracle_cache = {}


def _oracle(uplo, An, Bn):
    if uplo not in _oracle_cache:
        from oracle import native
        native.set_blas_threads(1)
        cores = os.cpu_count() or 1
        F, info = native.chol_tiled(An, NB, uplo, nthreads=cores)
        assert info == 0
        X = np.array(Bn, order='F', copy=True)
        native.ldiv_tiled(F, uplo, X, NB, nthreads=cores)
        _oracle_cache.clear()           # keep one uplo's factor in host memory
        _oracle_cache[uplo] = (F, X)
    return _oracle_cache[uplo]


def _berr(A, X, B):
    R = B - A @ X
    nA = A.abs().sum(dim=1).max()
    return float((R.abs().amax(dim=0) / (nA * X.abs().amax(dim=0) + B.abs().amax(dim=0))).max())


@pytest.mark.parametrize("engine", ["emulated", "dfma"])
@pytest.mark.parametrize("uplo", "UL")
def test_headline_class_vs_oracle(system, uplo, engine):
    import torch
    import dagger_gb300 as d
    A, B, An, Bn = system
    F, Xo = _oracle(uplo, An, Bn)
    old = d.set_f64_engine(engine)
    try:
        part = d.Blocks(NB, NB)
        C = d.cholesky(d.DArray.from_array(A, part), uplo)
        DB = d.DArray.from_array(B, part)
        d.ldiv_(C, DB)
        torch.cuda.synchronize()
        tri = torch.triu if uplo == 'U' else torch.tril
        G = tri(C.factors.collect())
        Ft = tri(torch.from_numpy(np.ascontiguousarray(F)).to(A.device))
        ef = float((G - Ft).abs().max() / Ft.abs().max())
        del G, Ft, C
        X = DB.collect()
        Xt = torch.from_numpy(np.ascontiguousarray(Xo)).to(A.device)
        ex = float((X - Xt).abs().max() / Xt.abs().max())
        bg, bo = _berr(A, X, B), _berr(A, Xt, B)
        print(f"N={N} uplo={uplo} engine={engine}: factor {ef:.2e}, solve {ex:.2e}, "
              f"backward error {bg:.2e} (oracle {bo:.2e})")
        assert ef <= FACTOR_TOL
        assert ex <= SOLVE_TOL
        assert bg <= 4 * bo + 1e-18
    finally:
        d.set_f64_engine(old)
