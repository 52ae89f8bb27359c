"""Batched persistent launch: many SPD systems of uneven size in one launch.

Each system is checked against the FP64 oracle (LAPACK solve of the same
seeded system): FP64 mode within 1e-13 relative per system (the systems are
well conditioned, kappa < 3), FP32+IR mode to a normwise backward error of
at most 1e-12 for every system.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _systems(count, nlo, nhi, seed):
    from oracle import tiled as o
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(nlo), math.log(nhi), count)).round().astype(int)
    rs = rng.integers(1, 9, count)
    As = [o.spd_uniform(int(n), seed * 1000 + i) for i, n in enumerate(ns)]
    Bs = [o.rhs_normal(int(n), int(r), seed * 1000 + i) for i, (n, r) in enumerate(zip(ns, rs))]
    return As, Bs


@pytest.mark.parametrize("mode", ["fp64", "fp32_ir"])
def test_batched_matches_oracle(mode):
    import torch
    import dagger_gb300 as d
    from dagger_gb300.batched import batched_solve
    from oracle import tiled as o
    As, Bs = _systems(60, 20, 700, 3)
    # include the bucket edges and a vector right-hand side
    extra = [(64, 1), (65, 8), (128, 3), (1024, 2), (1, 1)]
    for n, r in extra:
        As.append(o.spd_uniform(n, n))
        Bs.append(o.rhs_normal(n, r, n))
    tA = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in As]
    tB = [torch.from_numpy(np.ascontiguousarray(b)).cuda() for b in Bs]
    tB[-2] = tB[-2][:, 0]
    Xs, rep = batched_solve(tA, tB, mode=mode, tol=1e-12)
    assert rep["failed"] == 0 and all(i == 0 for i in rep["info"])
    for i, (A, B) in enumerate(zip(As, Bs)):
        X = Xs[i].cpu().numpy().reshape(B.shape[0], -1)
        Bm = B.reshape(B.shape[0], -1)
        if i == len(As) - 2:
            Bm = Bm[:, :1]
        ref = o.lapack_solve(A, Bm)
        if mode == "fp64":
            assert np.abs(X - ref).max() / np.abs(ref).max() <= 1e-13, i
        else:
            assert o.backward_error(A, X, Bm).max() <= 1e-12, i
            assert rep["backward_error"][i] <= 1e-12


def test_batched_reports_non_posdef():
    import torch
    from dagger_gb300.batched import batched_solve
    from oracle import tiled as o
    As = [o.spd_uniform(n, n) for n in (100, 200, 300)]
    As[1][50, 50] = -1000.0
    Bs = [o.rhs_normal(a.shape[0], 2, 1) for a in As]
    tA = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in As]
    tB = [torch.from_numpy(np.ascontiguousarray(b)).cuda() for b in Bs]
    _, rep = batched_solve(tA, tB, mode="fp64")
    assert rep["failed"] == 2 and rep["info"][1] > 0
    assert rep["info"][0] == 0 and rep["info"][2] == 0


def test_batched_widths_agree():
    """Panel widths 16 and 32 (the autotuner's choices) give the same answer."""
    import torch
    from dagger_gb300.batched import PackedBatch, batched_solve_packed
    As, Bs = _systems(20, 30, 300, 9)
    tA = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in As]
    tB = [torch.from_numpy(np.ascontiguousarray(b)).cuda() for b in Bs]
    outs = []
    for w in (16, 32):
        P = PackedBatch(tA, tB)
        batched_solve_packed(P, "fp64", widths=[w] * 5, ctas_per_sm=2)
        outs.append([P.solution(i).clone() for i in range(P.count)])
    for x16, x32 in zip(*outs):
        assert torch.allclose(x16, x32, rtol=1e-12, atol=1e-14)
