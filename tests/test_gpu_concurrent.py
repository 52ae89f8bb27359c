"""Whole calls from several host threads at once.

The reference runs every task on its own Julia task and stream
(ext/CUDAExt.jl:309-327), so a backend's entry points are called
concurrently.  The library gives each stream handle its own workspace for the
emulated FP64 engine and the LU (slice slots, panel buffers, pivots), grown in
stream order, and makes calls on the same stream handle take turns.  These
tests run two factor-and-solve pipelines (an N = 4096 Cholesky with the
emulated engine and its solve, then an N = 2048 pivoted LU and its solve) on
two threads at once, each on its own stream, and on two threads sharing the
default stream, and compare every output bit for bit with the same pipelines
run one after the other.
"""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_CHOL, N_LU, NB, NRHS = 4096, 2048, 512, 16


def _inputs(seed):
    from oracle import tiled as o
    r = np.random.default_rng(seed)
    A = o.spd_uniform(N_CHOL, seed)
    B = r.standard_normal((N_CHOL, NRHS))
    G = r.uniform(0.0, 1.0, (N_LU, N_LU))
    BL = r.standard_normal((N_LU, NRHS))
    return A, B, G, BL


def _pipeline(inp, stream):
    """cholesky, ldiv!, lu, ldiv! on `stream` (None: the default stream);
    returns the host copies of every output."""
    import torch
    import dagger_gb300 as d
    A, B, G, BL = inp
    ctx = torch.cuda.stream(stream) if stream is not None else torch.cuda.stream(
        torch.cuda.default_stream())
    with ctx:
        DA = d.DArray.from_array(A, d.Blocks(NB, NB))
        C = d.cholesky(DA)
        DB = d.DArray.from_array(B, d.Blocks(NB, NB))
        d.ldiv_(C, DB)
        DG = d.DArray.from_array(G, d.Blocks(NB, NB))
        F = d.lu(DG)
        DBL = d.DArray.from_array(BL, d.Blocks(NB, NB))
        d.ldiv_(F, DBL)
        out = (C.factors.numpy(), DB.numpy(), F.factors.numpy(), F.ipiv.cpu().numpy(),
               DBL.numpy())
    torch.cuda.current_stream().synchronize()
    return out


def _run_threads(inps, streams, rounds):
    results = [[None] * rounds for _ in inps]
    errors = []
    start = threading.Barrier(len(inps))

    def worker(i):
        try:
            import torch
            torch.cuda.set_device(0)
            for k in range(rounds):
                start.wait(timeout=120)
                results[i][k] = _pipeline(inps[i], streams[i])
        except BaseException as e:  # reported on the main thread
            errors.append(e)
            start.abort()

    ts = [threading.Thread(target=worker, args=(i,)) for i in range(len(inps))]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in ts), "a worker did not finish"
    if errors:
        raise errors[0]
    return results


@pytest.fixture(scope="module")
def serial():
    import dagger_gb300 as d
    old = d.set_f64_engine("emulated")
    try:
        inps = [_inputs(11), _inputs(12)]
        outs = [_pipeline(x, None) for x in inps]
        yield inps, outs
    finally:
        d.set_f64_engine(old)


def _check(outs, ref):
    names = ("cholesky factor", "cholesky solve", "lu factors", "ipiv", "lu solve")
    for got, want, name in zip(outs, ref, names):
        assert got.shape == want.shape, name
        assert np.array_equal(got, want), name


def test_serial_results_are_sound(serial):
    """The serial reference itself: factor residuals at FP64 accuracy."""
    inps, outs = serial
    for (A, B, G, BL), (U, X, LUf, piv, Y) in zip(inps, outs):
        U = np.triu(U)
        assert np.linalg.norm(U.T @ U - A) <= 1e-13 * np.linalg.norm(A)
        assert np.linalg.norm(A @ X - B) <= 1e-10 * np.linalg.norm(A) * np.linalg.norm(X)
        assert np.linalg.norm(G @ Y - BL) <= 1e-9 * np.linalg.norm(G) * np.linalg.norm(Y)
        assert piv.min() >= 1 and piv.max() <= N_LU


def test_two_threads_two_streams_bit_identical(serial):
    import torch
    import dagger_gb300 as d
    inps, ref = serial
    old = d.set_f64_engine("emulated")
    try:
        streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        res = _run_threads(inps, streams, rounds=3)
    finally:
        d.set_f64_engine(old)
    for i in range(2):
        for k in range(3):
            _check(res[i][k], ref[i])


def test_two_threads_one_stream_bit_identical(serial):
    """Both threads on the default stream: the calls take turns on the
    stream's workspace and still match the serial run."""
    import dagger_gb300 as d
    inps, ref = serial
    old = d.set_f64_engine("emulated")
    try:
        res = _run_threads(inps, [None, None], rounds=2)
    finally:
        d.set_f64_engine(old)
    for i in range(2):
        for k in range(2):
            _check(res[i][k], ref[i])


def test_release_memory_between_calls(serial):
    """dg_release_memory frees the idle per-stream workspaces; the next call
    allocates again and gives the same bits."""
    import torch
    import dagger_gb300 as d
    inps, ref = serial
    old = d.set_f64_engine("emulated")
    try:
        s = torch.cuda.Stream()
        a = _pipeline(inps[0], s)
        assert d.lib().dg_release_memory() == 0
        b = _pipeline(inps[0], s)
    finally:
        d.set_f64_engine(old)
    _check(a, ref[0])
    _check(b, ref[0])
