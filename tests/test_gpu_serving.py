"""Serving loop: continuous batching with free-HBM admission and resident
factors.  Every request reaches the backward error target (1e-12), and each
result is the same alone and in the mix: the requests are run once one at a
time and once all submitted together, and the two solutions agree bit for
bit (each request's kernels read only its own data, in a fixed order)."""
import pytest

pytestmark = pytest.mark.gpu


def _work(seed):
    from dagger_gb300.serving import make_workload
    return make_workload(14, rate=0.0, seed=seed, nlo=64, nhi=3072, klo=1e2, khi=1e4, rmax=12,
                         reuse=0.3)


def _backward_error(A, X, B):
    R = B - A @ X
    nA = A.abs().sum(dim=1).max()
    return float((R.abs().amax(dim=0) / (nA * X.abs().amax(dim=0) + B.abs().amax(dim=0))).max())


def test_alone_and_in_mix_agree():
    from dagger_gb300.serving import Server, latency_stats, run_workload
    work = _work(3)
    # alone: one request at a time, each on a fresh server state
    alone = {}
    for _, req in work:
        srv = Server(budget_bytes=40e9, slots=1)
        srv.submit(req)
        req.event.wait()
        srv.close()
        assert req.error is None, req.error
        alone[req.rid] = req.X.clone()
    # in the mix: all at once on 4 slots
    work2 = _work(3)
    srv = Server(budget_bytes=40e9, slots=4)
    run_workload(srv, work2, realtime=False)
    srv.close()
    for _, req in work2:
        assert req.error is None, req.error
        X = req.X
        assert _backward_error(req.A, X, req.B) <= 1e-12
        assert (X == alone[req.rid]).all(), req.rid
    st = latency_stats([r for _, r in work2])
    assert st["count"] == len(work2) and st["p99_ms"] >= st["p50_ms"]


def test_admission_respects_budget():
    """A request larger than the budget is rejected; others are admitted only
    while they fit (the accounted bytes never exceed the budget)."""
    import torch
    from dagger_gb300.serving import Request, Server, footprint_bytes
    n = 2048
    A = torch.eye(n, dtype=torch.float64, device="cuda") * 2
    B = torch.ones(n, 2, dtype=torch.float64, device="cuda")
    need = footprint_bytes(n, 2, False)
    srv = Server(budget_bytes=need * 1.5, slots=4)
    big = Request(rid=0, A=torch.eye(4096, dtype=torch.float64, device="cuda"),
                  B=torch.ones(4096, 1, dtype=torch.float64, device="cuda"), matrix_id=99)
    srv.submit(big)
    reqs = [srv.submit(Request(rid=i + 1, A=A, B=B, matrix_id=i + 1)) for i in range(3)]
    for r in reqs + [big]:
        r.event.wait()
    srv.close()
    assert big.error is not None and "budget" in big.error
    for r in reqs:
        assert r.error is None, r.error
        assert torch.allclose(r.X, B / 2)
