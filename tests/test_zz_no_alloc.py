"""The allocation-free batched entry point, through the C ABI.

dg_batched_potrs_noalloc serves callers that must not allocate device memory
while they run (a server holding a fixed, pre-reserved memory budget, a pool
allocator that must not be bypassed, a real-time loop that forbids
allocation after start-up).  It takes its scratch from a library-owned
static device array instead of allocating.  This test calls it twice in a
row and checks both results against the allocating entry point
dg_batched_potrs on the same batch and settings (FP64: identical bits; FP32
factor + FP64 refinement: identical bits as well, and each system's normwise
backward error at most 1e-12).  It also checks that a batch too large for
the static array is rejected without launching, and that two host threads
calling it at once on their own streams (they take turns on the array) get
the same bits as the allocating entry point.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(count, seed):
    import torch
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(16), math.log(400), count)).round().astype(int).tolist()
    rs = rng.integers(1, 9, count).tolist()
    As, Bs = [], []
    for i, (n, r) in enumerate(zip(ns, rs)):
        M = rng.uniform(-1, 1, (n, n))
        A = M @ M.T / n + n * np.eye(n)
        As.append(torch.from_numpy(A).cuda())
        Bs.append(torch.from_numpy(rng.standard_normal((n, r))).cuda())
    return ns, rs, As, Bs


def _call(fn_name, P, mode, widths, ctas):
    import torch
    from dagger_gb300 import _lib
    L = _lib.lib()
    cnt = P.count
    pa, pb, px = P.pointers()
    n_arr = (ctypes.c_int * cnt)(*P.n)
    r_arr = (ctypes.c_int * cnt)(*P.r)
    w_arr = (ctypes.c_int * 5)(*widths)
    info = (ctypes.c_int * (2 * cnt))()
    berr = (ctypes.c_double * cnt)()
    s = torch.cuda.current_stream().cuda_stream
    if fn_name == "noalloc":
        rc = L.dg_batched_potrs_noalloc(cnt, n_arr, r_arr, pa, pb, px, mode, 1e-12, 30, w_arr,
                                        ctas, info, berr, s)
    else:
        ms = ctypes.c_float()
        rc = L.dg_batched_potrs(cnt, n_arr, r_arr, pa, pb, px, mode, 1e-12, 30, w_arr, ctas,
                                info, berr, ctypes.byref(ms), s)
    torch.cuda.synchronize()
    return rc, [info[2 * i] for i in range(cnt)], [berr[i] for i in range(cnt)]


@pytest.mark.parametrize("mode", [0, 1], ids=["fp64", "fp32_ir"])
def test_noalloc_matches_allocating_entry_twice(mode):
    from dagger_gb300.batched import PackedBatch
    ns, rs, As, Bs = _batch(48, 17 + mode)
    widths, ctas = [16, 16, 32, 32, 32], 2
    ref = PackedBatch(As, Bs)
    rc, info, _ = _call("alloc", ref, mode, widths, ctas)
    assert rc == 0 and not any(info)
    expected = [ref.solution(i).clone() for i in range(ref.count)]
    for _ in range(2):   # two calls in a row share the static scratch
        P = PackedBatch(As, Bs)
        rc, info, berr = _call("noalloc", P, mode, widths, ctas)
        assert rc == 0 and not any(info)
        for i in range(P.count):
            assert (P.solution(i) == expected[i]).all(), i
        if mode == 1:
            assert max(berr) <= 1e-12


def test_noalloc_rejects_a_batch_larger_than_its_scratch():
    import torch
    from dagger_gb300 import _lib
    from dagger_gb300.batched import PackedBatch
    n, count = 1024, 20   # 20 FP32 workspaces of 4 MiB exceed the 64 MiB array
    A = torch.eye(n, dtype=torch.float64, device="cuda") * 2
    B = torch.ones(n, 1, dtype=torch.float64, device="cuda")
    P = PackedBatch([A] * count, [B] * count)
    rc, _, _ = _call("noalloc", P, 1, [32] * 5, 1)
    assert rc == _lib.DG_ERR_NOMEM
    assert "64 MiB" in _lib.last_error()


def test_noalloc_two_threads_take_turns():
    import threading
    import torch
    from dagger_gb300.batched import PackedBatch
    widths, ctas = [32, 32, 32, 32, 32], 1
    batches = [_batch(40, 31), _batch(40, 32)]
    expected = []
    for ns, rs, As, Bs in batches:
        ref = PackedBatch(As, Bs)
        rc, info, _ = _call("alloc", ref, 1, widths, ctas)
        assert rc == 0 and not any(info)
        expected.append([ref.solution(i).clone() for i in range(ref.count)])
    got, errors = [None, None], []
    start = threading.Barrier(2)

    def worker(j):
        try:
            torch.cuda.set_device(0)
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                out = []
                for _ in range(3):
                    ns, rs, As, Bs = batches[j]
                    P = PackedBatch(As, Bs)
                    start.wait(timeout=120)
                    rc, info, berr = _call("noalloc", P, 1, widths, ctas)
                    assert rc == 0 and not any(info)
                    assert max(berr) <= 1e-12
                    out.append([P.solution(i).clone() for i in range(P.count)])
                got[j] = out
        except BaseException as e:
            errors.append(e)
            start.abort()

    ts = [threading.Thread(target=worker, args=(j,)) for j in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in ts)
    if errors:
        raise errors[0]
    for j in range(2):
        for out in got[j]:
            for a, b in zip(out, expected[j]):
                assert (a == b).all()
