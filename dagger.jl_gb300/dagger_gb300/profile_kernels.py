"""Launches one hot kernel of the library a few times on a fixed workload, so
a profiler can capture exactly that kernel (ncu -k regex:<name> -c N).

    python -m dagger_gb300.profile_kernels gemm_f64   [--nb 1024] [--reps 4]
    python -m dagger_gb300.profile_kernels tc_gemm    [--m 8192] [--k 1024] [--terms 3]
    python -m dagger_gb300.profile_kernels trsm_f64   [--nb 1024]
    python -m dagger_gb300.profile_kernels batched    [--count 2000]
    python -m dagger_gb300.profile_kernels oz_gemm    [--m 8192] [--k 1024]
    python -m dagger_gb300.profile_kernels oz_slices  [--m 8192] [--k 1024]
    python -m dagger_gb300.profile_kernels lu_panel   [--m 32768] [--k 1024]
    python -m dagger_gb300.profile_kernels potrf_f64  [--nb 1024]
    python -m dagger_gb300.profile_kernels herm       [--m 8192] [--nb 1024]
    python -m dagger_gb300.profile_kernels diag       [--nb 1024]
    python -m dagger_gb300.profile_kernels tc6        [--m 8192] [--k 1024]
    python -m dagger_gb300.profile_kernels reblock    [--m 8192]
    python -m dagger_gb300.profile_kernels tc_f8      [--m 8192] [--k 1024]
    python -m dagger_gb300.profile_kernels lu_tiled   [--m 8192] [--nb 1024]
    python -m dagger_gb300.profile_kernels mixed      [--m 8192] [--nb 1024] [--prec fp32]

gemm_f64   the FP64 trailing-update tile GEMM of the plain path,
           C(nb x nb) -= A' B with nb x nb tiles (2 nb^3 flops per launch)
tc_gemm    the tcgen05 trailing SYRK/GEMM of the mixed form on an m x m
           output with K = k (2 m^2 k flops x terms per launch, BF16)
trsm_f64   the panel TRSM of one nb x nb tile
batched    the persistent batched launch on `count` systems, n in [32, 1024]
oz_gemm    the emulated FP64 GEMM (engine 2) on an m x m output with K = k:
           two split launches and one oz_gemm_kernel launch per call
           (2 m^2 k FP64 flops, 28 BF16 products of 2 m^2 k flops each)
oz_slices  oz_gemm_kernel alone on pre-cut slices, C(m x m) -= A'A with K = k
           (the launch bench.py's roofline times: the slices are cut once
           before the timed launches)
lu_panel   the pivoted panel factorization of the tiled LU (dg_getrf) on an
           m x k column-major matrix (uniform [0, 1), seed 5) with the emulated
           engine: 32-column leaf launches and the recursion's emulated
           updates; the matrix is restored before every call
potrf_f64  the FP64 factorization of one nb x nb diagonal tile (dg_potrf: 64 x 64
           potrf_base_kernel leaves, trsm_cols_kernel / trsm_base_kernel and
           the recursion's FP64 GEMMs)
herm       ishermitian on an m x m tile grid (herm_pair_kernel, one pass over A)
diag       the mixed form's FP32 factor + inverse of one nb x nb block
           (diag_chol_inv_kernel, one cooperative launch)
tc6        the FP32-accurate tensor-core product C(m x 64) = A'B, K = k, of the
           mixed form's solves (split3_kernel, tc_gemm_kernel<128, 6>)
reblock    copyto! between Blocks(1024, 1024) and Blocks(1000, 1000) of an m x m
           matrix (reblock_kernel; 16 bytes per element)
tc_f8      the FP8 product C(m x m) = A'A, K = k (dg_gemm_f8_tc_tn: e4m3_kernel,
           tc_gemm_persist_kernel<128, 1, true>; 2 m^2 k flops at the FP8 rate)
lu_tiled   lu!(A, RowMaximum()) of an m x m rand matrix, Blocks(nb, nb), emulated
           engine (dg_lu_tiled: leaves, lu_laswp_kernel, emulated updates); the
           matrix is restored before every call
mixed      the mixed factor of an m x m SPD matrix (G G'/m + I) with the given
           operand precision (fp32: gemm_fma<float> trailing updates)
Each prints the per-launch time measured with CUDA events.
"""
from __future__ import annotations

import argparse

import torch

from . import _lib
from .linalg import _stream


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["gemm_f64", "tc_gemm", "trsm_f64", "batched", "oz_gemm",
                                       "oz_slices", "lu_panel", "potrf_f64", "herm", "diag", "tc6",
                                       "reblock", "tc_f8", "lu_tiled", "mixed"])
    ap.add_argument("--nb", type=int, default=1024)
    ap.add_argument("--m", type=int, default=8192)
    ap.add_argument("--k", type=int, default=1024)
    ap.add_argument("--terms", type=int, default=3)
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--prec", default="fp32")
    a = ap.parse_args(argv)
    L = _lib.lib()
    s = _stream(None)
    dev = torch.device("cuda")
    if a.kernel == "lu_panel":
        from . import linalg
        old = linalg.set_f64_engine("emulated")
        g = torch.Generator(device=dev)
        g.manual_seed(5)
        A0 = torch.rand(a.k, a.m, generator=g, device=dev, dtype=torch.float64).t()
        A = torch.empty_strided((a.m, a.k), (1, a.m), dtype=torch.float64, device=dev)
        total = 0.0
        for _ in range(a.reps):
            A.copy_(A0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _, _, info = linalg.getrf_(A)
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        linalg.set_f64_engine(old)
        print(f"lu_panel m={a.m} k={a.k}: {total / a.reps:.2f} ms per panel (info {info})")
        return
    if a.kernel == "gemm_f64":
        nb = a.nb
        A, B, C = (torch.randn(nb, nb, dtype=torch.float64, device=dev) for _ in range(3))
        ms = _time(lambda: L.dg_gemm(b'T', b'N', nb, nb, nb, -1.0, A.data_ptr(), nb, B.data_ptr(),
                                     nb, 1.0, C.data_ptr(), nb, s), a.reps)
        print(f"gemm_f64 {nb}^3: {ms * 1e3:.1f} us/launch, {2 * nb ** 3 / ms / 1e9:.3f} TFLOP/s")
    elif a.kernel == "tc_gemm":
        m, k = a.m, a.k
        P = torch.randn(m, k, device=dev)
        hi = P.bfloat16()
        lo = (P - hi.float()).bfloat16()
        C = torch.zeros(m, m, device=dev)
        st = torch.zeros(1, dtype=torch.int32, device=dev)
        ms = _time(lambda: L.dg_gemm_tc_tn(m, m, k, a.terms, 0, hi.data_ptr(), lo.data_ptr(), k,
                                           hi.data_ptr(), lo.data_ptr(), k, -1.0, 1.0,
                                           C.data_ptr(), m, 128, st.data_ptr(), s), a.reps)
        fl = 2.0 * m * m * k * a.terms
        print(f"tc_gemm m={m} k={k} terms={a.terms}: {ms * 1e3:.1f} us/launch, "
              f"{fl / ms / 1e9:.1f} TFLOP/s")
    elif a.kernel == "oz_gemm":
        m, k = a.m, a.k
        A = torch.randn(m, k, dtype=torch.float64, device=dev)   # k x m column-major
        C = torch.randn(m, m, dtype=torch.float64, device=dev)
        ms = _time(lambda: L.dg_gemm_f64_emulated_tn(m, m, k, -1.0, A.data_ptr(), k, A.data_ptr(),
                                                     k, 1.0, C.data_ptr(), m, s), a.reps)
        fl = 2.0 * m * m * k
        print(f"oz_gemm m={m} k={k}: {ms * 1e3:.1f} us/call, {fl / ms / 1e9:.2f} FP64-equivalent "
              f"TFLOP/s, {28 * fl / ms / 1e9:.1f} BF16 TFLOP/s")
    elif a.kernel == "oz_slices":
        m, k = a.m, a.k
        ldk = (k + 7) // 8 * 8
        g = torch.Generator(device=dev)
        g.manual_seed(11)
        A = torch.randn(m, k, dtype=torch.float64, device=dev, generator=g)  # k x m column-major
        C = torch.randn(m, m, dtype=torch.float64, device=dev, generator=g)
        sl = torch.empty(7 * ldk * m, dtype=torch.bfloat16, device=dev)
        sc = torch.empty(m, dtype=torch.int64, device=dev)
        L.dg_f64_slices(k, m, A.data_ptr(), k, 1, sl.data_ptr(), ldk, sc.data_ptr(), s)
        ms = _time(lambda: L.dg_gemm_f64_slices(m, m, k, -1.0, sl.data_ptr(), ldk, sc.data_ptr(),
                                                sl.data_ptr(), ldk, sc.data_ptr(), 1.0,
                                                C.data_ptr(), m, None, s), a.reps)
        fl = 2.0 * m * m * k
        print(f"oz_slices m={m} k={k}: {ms * 1e3:.1f} us/launch, {fl / ms / 1e9:.2f} "
              f"FP64-equivalent TFLOP/s, {28 * fl / ms / 1e9:.1f} BF16 TFLOP/s")
    elif a.kernel == "trsm_f64":
        nb = a.nb
        T = torch.randn(nb, nb, dtype=torch.float64, device=dev) * 0.01
        T.diagonal().add_(1.0)
        B = torch.randn(nb, nb, dtype=torch.float64, device=dev)
        ms = _time(lambda: L.dg_trsm(b'L', b'U', b'T', b'N', nb, nb, 1.0, T.data_ptr(), nb,
                                     B.data_ptr(), nb, s), a.reps)
        print(f"trsm_f64 {nb}^2 x {nb}: {ms * 1e3:.1f} us/call, {nb ** 3 / ms / 1e9:.3f} TFLOP/s")
    elif a.kernel == "potrf_f64":
        nb = a.nb
        r = torch.rand(nb, nb, dtype=torch.float64, device=dev)
        S = r @ r.T / nb
        S.diagonal().add_(1.0)
        T = S.clone()
        import ctypes
        info = ctypes.c_int(0)

        def call():
            T.copy_(S)
            L.dg_potrf(b'U', nb, T.data_ptr(), nb, ctypes.byref(info), s)
        ms = _time(call, a.reps)
        print(f"potrf_f64 {nb}: {ms * 1e3:.1f} us/call (info {info.value})")
    elif a.kernel == "herm":
        from .darray import Blocks, DArray
        r = torch.rand(a.m, a.m, dtype=torch.float64, device=dev)
        D = DArray.from_array(r + r.T, Blocks(a.nb, a.nb))
        ms = _time(lambda: L.dg_ishermitian_tiled(a.m, a.nb, D.tile_ptrs(), s), a.reps)
        print(f"herm {a.m}: {ms * 1e3:.1f} us/call, {8.0 * a.m * a.m / ms / 1e6:.0f} GB/s")
    elif a.kernel == "diag":
        nb = a.nb
        r = torch.rand(nb, nb, device=dev)
        S = r @ r.T / nb
        S.diagonal().add_(1.0)
        M, V = S.clone(), torch.empty_like(S)
        import ctypes
        info = ctypes.c_int(0)

        def call():
            M.copy_(S)
            L.dg_potrf_inv_f32(nb, M.data_ptr(), nb, V.data_ptr(), nb, ctypes.byref(info), s)
        ms = _time(call, a.reps)
        print(f"diag {nb}: {ms * 1e3:.1f} us/call (info {info.value})")
    elif a.kernel == "tc_f8":
        m, k = a.m, a.k
        A = torch.randn(m, k, device=dev)
        C = torch.zeros(m, m, device=dev)
        ms = _time(lambda: L.dg_gemm_f8_tc_tn(m, m, k, -1.0, A.data_ptr(), k, A.data_ptr(), k,
                                              1.0, C.data_ptr(), m, s), a.reps)
        print(f"tc_f8 m={m} k={k}: {ms * 1e3:.1f} us/call (with the two conversions), "
              f"{2.0 * m * m * k / ms / 1e9:.1f} FP8 TFLOP/s")
    elif a.kernel == "lu_tiled":
        from . import linalg
        from .darray import Blocks, DArray
        old = linalg.set_f64_engine("emulated")
        g = torch.Generator(device=dev)
        g.manual_seed(5)
        A0 = torch.rand(a.m, a.m, generator=g, device=dev, dtype=torch.float64)
        D0 = DArray.from_array(A0, Blocks(a.nb, a.nb))
        DA = D0.copy()

        def call():
            DA.storage.copy_(D0.storage)
            linalg.lu_(DA, check_=False)
        ms = _time(call, a.reps)
        linalg.set_f64_engine(old)
        print(f"lu_tiled m={a.m} nb={a.nb}: {ms:.2f} ms/call, "
              f"{2.0 * a.m ** 3 / 3.0 / ms / 1e9:.2f} TFLOP/s")
    elif a.kernel == "mixed":
        from .darray import Blocks, DArray
        from .mixed import cholesky_mixed
        g = torch.Generator(device=dev)
        g.manual_seed(7)
        G = torch.randn(a.m, a.m, generator=g, device=dev, dtype=torch.float64)
        A = G @ G.T / a.m
        A.diagonal().add_(1.0)
        del G
        DA = DArray.from_array(A, Blocks(a.nb, a.nb))
        del A

        def call():
            cholesky_mixed(DA, a.prec, stream=torch.cuda.current_stream()).close()
        ms = _time(call, a.reps)
        print(f"mixed {a.prec} m={a.m}: {ms:.2f} ms per factorization, "
              f"{a.m ** 3 / 3.0 / ms / 1e9:.2f} TFLOP/s")
    elif a.kernel == "tc6":
        m, k, r = a.m, a.k, 64
        A = torch.randn(m, k, device=dev)
        B = torch.randn(r, k, device=dev)
        C = torch.zeros(r, m, device=dev)
        ms = _time(lambda: L.dg_gemm_f32_tc_tn(m, r, k, -1.0, A.data_ptr(), k, B.data_ptr(), k,
                                               1.0, C.data_ptr(), m, s), a.reps)
        print(f"tc6 m={m} n={r} k={k}: {ms * 1e3:.1f} us/call, "
              f"{6 * 2.0 * m * r * k / ms / 1e9:.1f} BF16 TFLOP/s")
    elif a.kernel == "reblock":
        from .darray import Blocks, DArray
        from .linalg import copy_reblock
        X = torch.randn(a.m, a.m, dtype=torch.float64, device=dev)
        S1 = DArray.from_array(X, Blocks(1024, 1024))
        S2 = DArray((a.m, a.m), Blocks(1000, 1000), device=dev)
        ms = _time(lambda: copy_reblock(S1, S2), a.reps)
        print(f"reblock {a.m}: {ms * 1e3:.1f} us/call, {16.0 * a.m * a.m / ms / 1e6:.0f} GB/s")
    else:
        from .autotune import sample_batch
        from .batched import PackedBatch, batched_solve_packed, flops
        As, Bs = sample_batch(a.count, 32, 1024, seed=1, device=dev)
        P = PackedBatch(As, Bs)
        for mode in ("fp64", "fp32_ir"):
            P.load_again()
            rep = batched_solve_packed(P, mode)
            fl = flops([x.shape[0] for x in As], [x.shape[1] for x in Bs])
            print(f"batched {mode} count={a.count}: {rep['elapsed_ms']:.1f} ms, "
                  f"{fl / rep['elapsed_ms'] / 1e9:.3f} TFLOP/s")


if __name__ == "__main__":
    main()
