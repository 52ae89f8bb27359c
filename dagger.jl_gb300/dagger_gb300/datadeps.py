"""spawn_datadeps / spawn with In, Out, InOut: the Dagger.jl datadeps API.

Mirrors `Dagger.spawn_datadeps(f)` (src/datadeps/queue.jl:35-106) and the
argument wrappers `In`, `Out`, `InOut`, `Deps` (src/datadeps/aliasing.jl:
165-181) for regions made of the tile calls of this path (potrf_, trsm_,
syrk_, gemm_, copyto_).  Inside a region, `spawn(f, args...)` records the
call; when the region ends, the tasks are handed to libdaggergb300, which
derives the dependencies with the datadeps rules, issues them on CUDA
streams joined by events inside a captured (and cached) CUDA graph, waits,
and rethrows the first failure: a PosDefException from a POTRF
(potrf_checked!, src/array/cholesky.jl:2-18) as the reference's region does
(queue.jl:79).

Unannotated arguments default to In, as in the reference.  Arguments that
are not tensors (characters, scalars) are passed through.

Example, the reference's raw datadeps Cholesky (test/datadeps.jl:960-975):

    with spawn_datadeps():
        for k in range(mt):
            spawn(potrf_, 'L', InOut(M[k][k]))
            for m in range(k + 1, mt):
                spawn(trsm_, 'R', 'L', 'T', 'N', 1.0, In(M[k][k]), InOut(M[m][k]))
            ...
"""
from __future__ import annotations

import ctypes
import threading

import torch

from . import linalg as _la
from ._lib import (DG_IN, DG_INOUT, DG_OP_COPY, DG_OP_GEMM, DG_OP_POTRF, DG_OP_SYRK, DG_OP_TRSM,
                   DG_OUT, DgTask, PosDefException, ch, check, lib)


class In:
    """Read-only dependency."""

    def __init__(self, x):
        self.x = x


class Out:
    """Write-only dependency."""

    def __init__(self, x):
        self.x = x


class InOut:
    """Read-write dependency."""

    def __init__(self, x):
        self.x = x


def _unwrap(a):
    if isinstance(a, (In, Out, InOut)):
        mode = DG_IN if isinstance(a, In) else DG_OUT if isinstance(a, Out) else DG_INOUT
        return a.x, mode
    return a, 0


def copyto_(dest: torch.Tensor, src: torch.Tensor):
    """copyto!(dest, src) on equally shaped tiles."""
    dest.copy_(src)
    return dest


_tls = threading.local()


class DataDepsRegion:
    """One datadeps region: the recorded tasks and the tensors they keep alive."""

    def __init__(self, use_graph: bool = True, serial: bool = False, stream=None):
        self.use_graph = use_graph
        self.serial = serial
        self.stream = stream
        self.handle = lib().dg_region_create()
        self.keep = []
        self.ntasks = 0

    def _add(self, t: DgTask, tensors):
        self.keep.extend(tensors)
        check(lib().dg_region_add(self.handle, ctypes.byref(t)))
        self.ntasks += 1

    def record(self, fn, args):
        vals, modes = zip(*[_unwrap(a) for a in args]) if args else ((), ())
        t = DgTask()
        if fn is _la.potrf_:
            uplo, A = vals[0], vals[1]
            p, r, c, ld = _la._colmajor(A, "A")
            t.op, t.uplo, t.n, t.c, t.ldc = DG_OP_POTRF, ch(uplo), r, p, ld
            t.mode_c = modes[1] or DG_IN
            self._add(t, [A])
        elif fn is _la.trsm_:
            side, uplo, transa, diag, alpha, A, B = vals
            pa, _, _, lda = _la._colmajor(A, "A")
            pb, m, n, ldb = _la._colmajor(B, "B")
            t.op, t.side, t.uplo, t.transa, t.diag = DG_OP_TRSM, ch(side), ch(uplo), ch(transa), ch(diag)
            t.m, t.n, t.alpha, t.a, t.lda, t.c, t.ldc = m, n, float(alpha), pa, lda, pb, ldb
            t.mode_a, t.mode_c = modes[5] or DG_IN, modes[6] or DG_IN
            self._add(t, [A, B])
        elif fn is _la.syrk_:
            uplo, trans, alpha, A, beta, C = vals
            pa, ra, ca, lda = _la._colmajor(A, "A")
            pc, n, _, ldc = _la._colmajor(C, "C")
            t.op, t.uplo, t.trans = DG_OP_SYRK, ch(uplo), ch(trans)
            t.n, t.k = n, (ca if trans in ('N', 'n') else ra)
            t.alpha, t.beta, t.a, t.lda, t.c, t.ldc = float(alpha), float(beta), pa, lda, pc, ldc
            t.mode_a, t.mode_c = modes[3] or DG_IN, modes[5] or DG_IN
            self._add(t, [A, C])
        elif fn is _la.gemm_:
            ta, tb, alpha, A, B, beta, C = vals
            pa, ra, ca, lda = _la._colmajor(A, "A")
            pb, _, _, ldb = _la._colmajor(B, "B")
            pc, m, n, ldc = _la._colmajor(C, "C")
            t.op, t.transa, t.transb = DG_OP_GEMM, ch(ta), ch(tb)
            t.m, t.n, t.k = m, n, (ca if ta in ('N', 'n') else ra)
            t.alpha, t.beta = float(alpha), float(beta)
            t.a, t.lda, t.b, t.ldb, t.c, t.ldc = pa, lda, pb, ldb, pc, ldc
            t.mode_a, t.mode_b, t.mode_c = modes[3] or DG_IN, modes[4] or DG_IN, modes[6] or DG_IN
            self._add(t, [A, B, C])
        elif fn is copyto_:
            D, S = vals
            pd, m, n, ldd = _la._colmajor(D, "dest")
            ps, _, _, lds = _la._colmajor(S, "src")
            t.op, t.m, t.n, t.a, t.lda, t.c, t.ldc = DG_OP_COPY, m, n, ps, lds, pd, ldd
            t.mode_a, t.mode_c = modes[1] or DG_IN, modes[0] or DG_IN
            self._add(t, [D, S])
        else:
            raise NotImplementedError(
                f"{getattr(fn, '__name__', fn)} is not a tile call of this path "
                "(potrf_, trsm_, syrk_, gemm_, copyto_)")

    def stats(self):
        nt, ne = ctypes.c_int(0), ctypes.c_int(0)
        check(lib().dg_region_stats(self.handle, ctypes.byref(nt), ctypes.byref(ne)))
        return nt.value, ne.value

    def edges(self):
        """[(task, predecessor), ...] derived by the datadeps rules."""
        _, ne = self.stats()
        buf = (ctypes.c_int * (2 * max(ne, 1)))()
        n = lib().dg_region_edges(self.handle, buf, ne)
        return [(buf[2 * i], buf[2 * i + 1]) for i in range(n)]

    def run(self):
        rc = lib().dg_region_run(self.handle, int(self.use_graph), int(self.serial),
                                 _la._stream(self.stream))
        if rc < 0:
            check(rc)
        return rc

    def close(self):
        if self.handle:
            lib().dg_region_destroy(self.handle)
            self.handle = None
        self.keep = []


class spawn_datadeps:
    """Context manager (and decorator-style callable) for a datadeps region.

        with spawn_datadeps():
            spawn(gemm_, 'T', 'N', -1.0, In(a), In(b), 1.0, InOut(c))

    or spawn_datadeps(f) which calls f() inside a region and returns its result.
    On exit the region runs to completion; a failed POTRF raises
    PosDefException(info)."""

    def __new__(cls, f=None, *, use_graph: bool = True, serial: bool = False, stream=None):
        self = super().__new__(cls)
        self.region = None
        self.opts = dict(use_graph=use_graph, serial=serial, stream=stream)
        if f is not None:
            with self:
                result = f()
            return result
        return self

    def __enter__(self):
        self.prev = getattr(_tls, "region", None)
        self.region = DataDepsRegion(**self.opts)
        _tls.region = self.region
        return self.region

    def __exit__(self, et, ev, tb):
        _tls.region = self.prev
        try:
            if et is None:
                info = self.region.run()
                if info > 0:
                    raise PosDefException(info)
        finally:
            self.region.close()
        return False


def spawn(fn, *args):
    """Dagger.@spawn inside a datadeps region: record; outside: run now."""
    region = getattr(_tls, "region", None)
    if region is None:
        return fn(*[_unwrap(a)[0] for a in args])
    region.record(fn, args)
    return None
