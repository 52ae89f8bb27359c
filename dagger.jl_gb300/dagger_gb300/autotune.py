"""Autotuner for the batched persistent launch.

For each dtype mode ("fp64", "fp32_ir") and size bucket (n <= 64, 128, 256,
512, 1024) it times the persistent kernel on a seeded sample batch drawn from
that bucket with each candidate panel width (16, 32), then the grid
multiplier (CTAs per SM: 1, 2, 3) on a mixed-size sample, and stores the
fastest choices in autotune_table.json next to this file:

    {"fp64": {"w": {"64": 16, ...}, "ctas_per_sm": 2, "ms": {...}},
     "fp32_ir": {...}, "device": "...", "sm_count": 152}

Run:  python -m dagger_gb300.autotune   (needs a GPU)
"""
from __future__ import annotations

import json
import math
import sys

import torch

from .batched import BUCKET_EDGES, TABLE, PackedBatch, batched_solve_packed


def sample_batch(count, nlo, nhi, seed, device, rmax=8):
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    u = torch.rand(count, generator=g, dtype=torch.float64)
    ns = [max(nlo, min(nhi, int(round(math.exp(math.log(nlo) + x * (math.log(nhi) - math.log(nlo)))))))
          for x in u.tolist()]
    rs = [1 + int(x) for x in (torch.rand(count, generator=g) * rmax).tolist()]
    gd = torch.Generator(device=device)
    gd.manual_seed(seed)
    As, Bs = [], []
    for n, r in zip(ns, rs):
        Bm = torch.rand(n, n, device=device, dtype=torch.float64, generator=gd) * 2 - 1
        A = Bm @ Bm.T / n
        A.diagonal().add_(n)
        As.append(A)
        Bs.append(torch.randn(n, r, device=device, dtype=torch.float64, generator=gd))
    return As, Bs


def _time(P, mode, widths, ctas, reps=2):
    best = None
    for _ in range(reps):
        P.load_again()  # the FP64 mode factors in place: every run starts from the inputs
        rep = batched_solve_packed(P, mode, widths=widths, ctas_per_sm=ctas)
        best = rep["elapsed_ms"] if best is None else min(best, rep["elapsed_ms"])
    return best


def tune(device="cuda", per_bucket=None, verbose=True):
    table = {"device": torch.cuda.get_device_name(), "sm_count":
             torch.cuda.get_device_properties(0).multi_processor_count}
    sms = table["sm_count"]
    for mode in ("fp64", "fp32_ir"):
        widths = {}
        ms = {}
        lo = 16
        for e in BUCKET_EDGES:
            cnt = per_bucket or max(sms, min(4 * sms, int(4e7 / e ** 2)))
            As, Bs = sample_batch(cnt, max(lo, 8), e, seed=e, device=device)
            best_w, best_t = 32, None
            for w in (16, 32):
                P = PackedBatch(As, Bs)
                t = _time(P, mode, [w] * 5, 1 if mode == "fp32_ir" else 2)
                ms[f"{e}:w{w}"] = t
                if best_t is None or t < best_t:
                    best_w, best_t = w, t
            widths[str(e)] = best_w
            lo = e + 1
            if verbose:
                print(f"[{mode}] n<={e}: w={best_w} ({best_t:.2f} ms)", file=sys.stderr)
        As, Bs = sample_batch(per_bucket or 2 * sms, 32, 1024, seed=99, device=device)
        wl = [widths[str(e)] for e in BUCKET_EDGES]
        best_c, best_t = 1, None
        for c in (1, 2, 3):
            P = PackedBatch(As, Bs)
            t = _time(P, mode, wl, c)
            ms[f"ctas{c}"] = t
            if best_t is None or t < best_t:
                best_c, best_t = c, t
        table[mode] = {"w": widths, "ctas_per_sm": best_c, "ms": ms}
        if verbose:
            print(f"[{mode}] ctas_per_sm={best_c}", file=sys.stderr)
    return table


def main():
    table = tune()
    with open(TABLE, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    print(json.dumps(table))


if __name__ == "__main__":
    main()
