"""The C ABI library: loads, exports every declared symbol, and its
datadeps engine derives the reference's dependencies (host-only, no GPU).

The region calls used here (create/add/stats/edges/destroy) only record
tasks and compute dependencies: they touch no device memory, so fake
pointers are fine and no CUDA context is created.
"""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    from dagger_gb300 import _lib
    L = _lib.lib()
    declared = _declared()
    assert len(declared) >= 20
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert declared <= set(_lib.SIGNATURES), sorted(declared - set(_lib.SIGNATURES))


def test_version_and_error_strings():
    from dagger_gb300 import _lib
    assert b"sm_103a" in _lib.lib().dg_version()
    assert isinstance(_lib.last_error(), str)


def _cholesky_region(mt, nb, uplo, base=0x10000000):
    """Records _chol!'s task loop with fake tile pointers; returns the region."""
    from dagger_gb300 import _lib
    L = _lib.lib()
    r = L.dg_region_create()
    slot = nb * nb * 8
    ptr = lambda i, j: base + (i + j * mt) * slot  # noqa: E731
    from oracle.tiled import chol_tasks
    for kind, reads, writes in chol_tasks(mt, uplo):
        t = _lib.DgTask()
        (wi, wj), = writes
        if kind == 'potrf':
            t.op, t.uplo, t.n, t.c, t.ldc = _lib.DG_OP_POTRF, uplo.encode(), nb, ptr(wi, wj), nb
        elif kind == 'trsm':
            (ai, aj), = reads
            t.op, t.side, t.uplo, t.transa, t.diag = _lib.DG_OP_TRSM, (b'L' if uplo == 'U' else b'R'), uplo.encode(), b'T', b'N'
            t.m = t.n = nb
            t.alpha, t.a, t.lda, t.c, t.ldc = 1.0, ptr(ai, aj), nb, ptr(wi, wj), nb
        elif kind == 'syrk':
            (ai, aj), = reads
            t.op, t.uplo, t.trans, t.n, t.k = _lib.DG_OP_SYRK, uplo.encode(), (b'T' if uplo == 'U' else b'N'), nb, nb
            t.alpha, t.beta, t.a, t.lda, t.c, t.ldc = -1.0, 1.0, ptr(ai, aj), nb, ptr(wi, wj), nb
        else:
            (ai, aj), (bi, bj) = reads
            t.op = _lib.DG_OP_GEMM
            t.transa, t.transb = (b'T', b'N') if uplo == 'U' else (b'N', b'T')
            t.m = t.n = t.k = nb
            t.alpha, t.beta = -1.0, 1.0
            t.a, t.lda, t.b, t.ldb, t.c, t.ldc = ptr(ai, aj), nb, ptr(bi, bj), nb, ptr(wi, wj), nb
        assert L.dg_region_add(r, ctypes.byref(t)) == 0
    return r


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("mt", [1, 2, 5, 8])
def test_native_datadeps_matches_rules(uplo, mt):
    """Edges derived natively == the datadeps rules applied by the oracle."""
    from dagger_gb300 import _lib
    from oracle.tiled import chol_tasks, datadeps_edges
    L = _lib.lib()
    r = _cholesky_region(mt, 64, uplo)
    nt, ne = ctypes.c_int(), ctypes.c_int()
    L.dg_region_stats(r, ctypes.byref(nt), ctypes.byref(ne))
    tasks = chol_tasks(mt, uplo)
    assert nt.value == len(tasks)
    buf = (ctypes.c_int * (2 * max(ne.value, 1)))()
    n = L.dg_region_edges(r, buf, ne.value)
    got = {}
    for i in range(n):
        got.setdefault(buf[2 * i], set()).add(buf[2 * i + 1])
    want = datadeps_edges(tasks)
    for t in range(len(tasks)):
        assert got.get(t, set()) == want[t], (t, tasks[t])
    L.dg_region_destroy(r)


def test_task_counts_match_reference():
    """120 tasks at N=4096/512 and 5984 at 32768/1024 (POTRF mt, TRSM and
    SYRK mt(mt-1)/2, GEMM C(mt,3))."""
    from oracle.tiled import chol_tasks
    assert len(chol_tasks(8)) == 120
    assert len(chol_tasks(32)) == 5984


def test_strided_overlap():
    """Tiles viewed inside one column-major matrix (ld = N) alias only where
    their rows and columns meet (the reference's StridedAliasing)."""
    from dagger_gb300 import _lib
    L = _lib.lib()
    N, nb = 256, 64
    base = 0x20000000

    def tile(i, j):
        return base + (i * nb + j * nb * N) * 8

    r = L.dg_region_create()

    def gemm(c_i, c_j, a, b):
        t = _lib.DgTask()
        t.op, t.transa, t.transb = _lib.DG_OP_GEMM, b'N', b'N'
        t.m = t.n = t.k = nb
        t.alpha, t.beta = 1.0, 1.0
        t.a, t.lda, t.b, t.ldb, t.c, t.ldc = tile(*a), N, tile(*b), N, tile(c_i, c_j), N
        assert L.dg_region_add(r, ctypes.byref(t)) == 0

    gemm(0, 0, (3, 3), (3, 2))   # task 0 writes tile (0,0)
    gemm(1, 0, (3, 3), (3, 2))   # task 1 writes (1,0): same columns, other rows
    gemm(0, 1, (3, 3), (3, 2))   # task 2 writes (0,1): other columns
    gemm(2, 2, (0, 0), (1, 0))   # task 3 reads (0,0) and (1,0)
    gemm(1, 0, (0, 1), (3, 3))   # task 4 writes (1,0), reads (0,1)
    buf = (ctypes.c_int * 64)()
    n = L.dg_region_edges(r, buf, 32)
    edges = {(buf[2 * i], buf[2 * i + 1]) for i in range(n)}
    assert edges == {(3, 0), (3, 1), (4, 1), (4, 2), (4, 3)}
    L.dg_region_destroy(r)


def test_invalid_arguments_are_reported_without_a_gpu():
    """Argument checks run before any CUDA call: -i for argument i."""
    from dagger_gb300 import _lib
    L = _lib.lib()
    assert L.dg_gemm(b'X', b'N', 1, 1, 1, 1.0, None, 1, None, 1, 0.0, None, 1, None) == -1
    assert L.dg_trsm(b'L', b'U', b'N', b'N', 4, 4, 1.0, None, 2, None, 4, None) == -9
    assert L.dg_syrk(b'U', b'T', -1, 1, 1.0, None, 1, 0.0, None, 1, None) == -3
    assert L.dg_cholesky_tiled(b'Q', 4, 2, None, None) == -1
    assert "invalid argument" in _lib.last_error()


def test_invalid_arguments_of_the_newer_entry_points():
    """The tensor-core building blocks, the LU and the checks validate their
    arguments before any CUDA call as well."""
    from dagger_gb300 import _lib
    L = _lib.lib()
    # m < 0, lda < k, ldb < k, ldc < m
    assert L.dg_gemm_f8_tc_tn(-1, 4, 16, 1.0, None, 16, None, 16, 0.0, None, 1, None) == -1
    assert L.dg_gemm_f8_tc_tn(4, 4, 16, 1.0, None, 8, None, 16, 0.0, None, 4, None) == -6
    assert L.dg_gemm_f8_tc_tn(4, 4, 16, 1.0, None, 16, None, 8, 0.0, None, 4, None) == -8
    assert L.dg_gemm_f8_tc_tn(4, 4, 16, 1.0, None, 16, None, 16, 0.0, None, 2, None) == -11
    # empty products do nothing and succeed
    assert L.dg_gemm_f8_tc_tn(0, 4, 16, 1.0, None, 16, None, 16, 0.0, None, 1, None) == 0
    assert L.dg_gemm_f32_tc_tn(-1, 4, 16, 1.0, None, 16, None, 16, 0.0, None, 1, None) == -1
    # LU: nb <= 0, a pivot flag other than 0 / 1
    assert L.dg_lu_tiled(4, 4, 0, None, 1, None, None) == -3
    assert L.dg_lu_tiled(4, 4, 2, None, 2, None, None) == -5
    # chkfinite of an m x n grid: mb <= 0
    assert L.dg_chkfinite_tiled_mn(4, 4, 0, 2, None, None) == -3
    assert L.dg_ishermitian_tiled(-1, 2, None, None) == -1


def test_tile_local_info():
    """The reference's info (the failing tile's own LAPACK info) from the
    global order the library reports."""
    import dagger_gb300 as d
    assert d.tile_local_info(0, 64) == 0
    assert d.tile_local_info(1, 64) == 1
    assert d.tile_local_info(64, 64) == 64
    assert d.tile_local_info(65, 64) == 1
    assert d.tile_local_info(200, 64) == 8
    assert d.tile_local_info(130, 128) == 2
