"""Many independent SPD systems factored and solved in one persistent launch.

    X, report = batched_solve(As, Bs, mode="fp64" | "fp32_ir", tol=1e-12)

As[i] is an n_i x n_i SPD CUDA tensor (n_i <= 1024), Bs[i] an n_i or
n_i x r_i tensor (r_i <= 8).  The systems are copied into one packed device
buffer (column-major per system), sorted into size buckets and handed to
dg_batched_potrs, which runs every factorization and solve in a single
launch.  "fp64" factors and solves in FP64; "fp32_ir" factors in FP32 and
refines in FP64 to a normwise backward error of at most `tol`.  Each size
bucket's panel width and the grid per SM come from the autotuner's table
(autotune.py) for this dtype when present.
"""
from __future__ import annotations

import ctypes
import json
import os

import torch

from ._lib import check, lib
from .linalg import _stream

BUCKET_EDGES = (64, 128, 256, 512, 1024)
TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "autotune_table.json")


def load_table():
    try:
        with open(TABLE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def config_for(mode: str, table: dict | None = None):
    """(bucket widths, ctas per SM) for a mode from the autotune table."""
    t = (table if table is not None else load_table()).get(mode, {})
    widths = [int(t.get("w", {}).get(str(e), 32)) for e in BUCKET_EDGES]
    return widths, int(t.get("ctas_per_sm", 2 if mode == "fp64" else 1))


class PackedBatch:
    """Device-resident packed copies of a batch (one allocation per array kind)."""

    def __init__(self, As, Bs, device=None):
        self.count = len(As)
        self.n = [int(a.shape[0]) for a in As]
        self.r = [1 if b.dim() == 1 else int(b.shape[1]) for b in Bs]
        dev = device or As[0].device
        offA, offB = [], []
        sa = sb = 0
        for n, r in zip(self.n, self.r):
            offA.append(sa)
            offB.append(sb)
            sa += (n * n + 31) // 32 * 32
            sb += (n * r + 31) // 32 * 32
        self.A = torch.empty(max(sa, 1), dtype=torch.float64, device=dev)
        self.B = torch.empty(max(sb, 1), dtype=torch.float64, device=dev)
        self.X = torch.empty(max(sb, 1), dtype=torch.float64, device=dev)
        self.offA, self.offB = offA, offB
        self.load(As, Bs)

    def load(self, As, Bs):
        for i, (a, b) in enumerate(zip(As, Bs)):
            n, r = self.n[i], self.r[i]
            # column-major copies: A^T row-major == A column-major
            self.A[self.offA[i]:self.offA[i] + n * n].view(n, n).copy_(a.T)
            bb = b.reshape(n, r)
            self.B[self.offB[i]:self.offB[i] + n * r].view(r, n).copy_(bb.T)
        self._A0 = None

    def load_again(self):
        """Restores the matrices after an FP64 run (which factors them in place)."""
        if self._A0 is None:
            self._A0 = self.A.clone()
        else:
            self.A.copy_(self._A0)

    def pointers(self):
        es = 8
        pa = (ctypes.c_void_p * self.count)(*[self.A.data_ptr() + o * es for o in self.offA])
        pb = (ctypes.c_void_p * self.count)(*[self.B.data_ptr() + o * es for o in self.offB])
        px = (ctypes.c_void_p * self.count)(*[self.X.data_ptr() + o * es for o in self.offB])
        return pa, pb, px

    def solution(self, i):
        n, r = self.n[i], self.r[i]
        return self.X[self.offB[i]:self.offB[i] + n * r].view(r, n).T


def batched_solve_packed(P: PackedBatch, mode: str = "fp64", tol: float = 1e-12,
                         max_iter: int = 30, widths=None, ctas_per_sm=None, stream=None):
    """Runs the persistent launch on a PackedBatch; returns a report dict."""
    if mode not in ("fp64", "fp32_ir"):
        raise ValueError("mode must be 'fp64' or 'fp32_ir'")
    w0, c0 = config_for(mode)
    widths = widths or w0
    ctas = ctas_per_sm or c0
    cnt = P.count
    n_arr = (ctypes.c_int * cnt)(*P.n)
    r_arr = (ctypes.c_int * cnt)(*P.r)
    pa, pb, px = P.pointers()
    w_arr = (ctypes.c_int * 5)(*widths)
    info = (ctypes.c_int * (2 * cnt))()
    berr = (ctypes.c_double * cnt)()
    ms = ctypes.c_float(0)
    rc = lib().dg_batched_potrs(cnt, n_arr, r_arr, pa, pb, px, 0 if mode == "fp64" else 1,
                                float(tol), int(max_iter), w_arr, int(ctas), info, berr,
                                ctypes.byref(ms), _stream(stream))
    if rc < 0:
        check(rc)
    return {"failed": rc, "elapsed_ms": ms.value,
            "info": [info[2 * i] for i in range(cnt)],
            "iterations": [info[2 * i + 1] for i in range(cnt)],
            "backward_error": [berr[i] for i in range(cnt)] if mode == "fp32_ir" else None,
            "widths": list(widths), "ctas_per_sm": ctas}


def batched_solve(As, Bs, mode: str = "fp64", tol: float = 1e-12, max_iter: int = 30,
                  stream=None):
    """Solves As[i] X_i = Bs[i] for every i in one launch.  Returns (Xs, report)."""
    P = PackedBatch(As, Bs)
    rep = batched_solve_packed(P, mode, tol, max_iter, stream=stream)
    Xs = []
    for i, b in enumerate(Bs):
        x = P.solution(i)
        Xs.append(x[:, 0] if b.dim() == 1 else x)
    return Xs, rep


def flops(ns, rs, mode="fp64"):
    """Algorithmic flops of a batch: n^3/3 + 2 n^2 r per system."""
    return sum(n ** 3 / 3.0 + 2.0 * n * n * r for n, r in zip(ns, rs))
