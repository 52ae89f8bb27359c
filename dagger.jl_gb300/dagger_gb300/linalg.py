"""The reference-facing API of the Cholesky factor-and-solve path.

Python mirror of what Dagger.jl exposes for this path, with the same names,
argument meanings and error behaviour:

  cholesky(DA, uplo)   LinearAlgebra.cholesky on a DArray: cholcopy then the
                       tiled factor (src/array/cholesky.jl:1,19-108)
  cholesky_(DA, uplo)  cholesky! (in place)
  lu(DA, pivot) / lu_  LinearAlgebra.lu / lu! with RowMaximum or NoPivot
                       (src/array/lu.jl); ldiv(F, B) / ldiv_(F, B) with an LU
                       (linalg.jl:221-308); getrf_ the panel's LAPACK call
  ldiv_(C, B)          ldiv!(C::Cholesky{T,<:DMatrix}, B) (src/array/linalg.jl:352-405)
  ishermitian / issymmetric on a DArray (linalg.jl:43-124)
  potrf_, trsm_, syrk_, gemm_, trsv_, gemv_
                       the BLAS/LAPACK tile calls the reference substitutes
                       with CUBLAS/CUSOLVER (ext/CUDAExt.jl:329-348), on
                       column-major torch CUDA tensors

Every compute call goes through libdaggergb300 (C ABI); none has a CPU path.
A matrix that is not positive definite raises PosDefException(info) from
cholesky / cholesky_ (potrf_checked!, cholesky.jl:2-18), or returns info
with check=False (cholesky(A; check=false) in LinearAlgebra); info is the
global order of the failing leading minor (tile_local_info gives the tile's
own number, which the reference records).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import PosDefException, ch, check, lib
from .darray import Blocks, DArray


def tile_local_info(info: int, nb: int) -> int:
    """The LAPACK info of the failing diagonal tile, as potrf_checked!
    (cholesky.jl:2-18) records it and _chol! returns it, from the global
    order of the first leading minor that is not positive definite (what
    cholesky / cholesky_ report, as LinearAlgebra's dense cholesky does).
    Tiles are Blocks(nb, nb); info <= 0 is returned unchanged."""
    if nb <= 0:
        raise ValueError("nb must be positive")
    return info if info <= 0 else info - nb * ((info - 1) // nb)


def _stream(stream=None) -> int:
    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


def _colmajor(t: torch.Tensor, name: str):
    """(pointer, rows, cols, ld) of a column-major FP64 CUDA tensor (a tile)."""
    if not t.is_cuda or t.dtype != torch.float64:
        raise TypeError(f"{name} must be a float64 CUDA tensor")
    if t.dim() == 1:
        return t.data_ptr(), t.shape[0], 1, max(t.shape[0], 1)
    r, c = t.shape
    if t.stride(0) != 1 and not (c == 1):
        raise ValueError(f"{name} must be column-major (stride(0) == 1)")
    ld = t.stride(1) if c > 1 else max(r, 1)
    return t.data_ptr(), r, c, max(ld, 1)


# ---------------------------------------------------------------------------
# tile calls (BLAS / LAPACK conventions)
# ---------------------------------------------------------------------------

def potrf_(uplo: str, A: torch.Tensor, stream=None):
    """LAPACK.potrf!(uplo, A) -> (A, info); synchronises like the reference's."""
    p, r, c, ld = _colmajor(A, "A")
    if r != c:
        raise ValueError("potrf_: A must be square")
    info = ctypes.c_int(0)
    rc = lib().dg_potrf(ch(uplo), r, p, ld, ctypes.byref(info), _stream(stream))
    if rc < 0:
        check(rc)
    return A, info.value


def getrf_(A: torch.Tensor, stream=None):
    """LAPACK.getrf!(A) -> (A, ipiv, info) on a column-major CUDA tensor: the
    pivoted LU in place, ipiv a 1-based int64 CUDA tensor of min(m, n) rows;
    synchronises like the reference's getrf!.  The panel task of
    lu!(A, RowMaximum()) (factor_panel_lapack!, lu.jl:263-304)."""
    p, r, c, ld = _colmajor(A, "A")
    ipiv = torch.empty(max(min(r, c), 1), dtype=torch.int64, device=A.device)
    info = ctypes.c_int(0)
    rc = lib().dg_getrf(r, c, p, ld, ipiv.data_ptr(), ctypes.byref(info), _stream(stream))
    if rc < 0:
        check(rc)
    return A, ipiv[:min(r, c)], info.value


def trsm_(side, uplo, transa, diag, alpha, A, B, stream=None):
    """BLAS.trsm!(side, uplo, transa, diag, alpha, A, B) -> B."""
    pa, ra, ca, lda = _colmajor(A, "A")
    pb, m, n, ldb = _colmajor(B, "B")
    check(lib().dg_trsm(ch(side), ch(uplo), ch(transa), ch(diag), m, n, float(alpha), pa, lda,
                        pb, ldb, _stream(stream)))
    return B


def syrk_(uplo, trans, alpha, A, beta, C, stream=None):
    """BLAS.syrk!(uplo, trans, alpha, A, beta, C) -> C."""
    pa, ra, ca, lda = _colmajor(A, "A")
    pc, n, n2, ldc = _colmajor(C, "C")
    k = ca if trans in ('N', 'n') else ra
    check(lib().dg_syrk(ch(uplo), ch(trans), n, k, float(alpha), pa, lda, float(beta), pc, ldc,
                        _stream(stream)))
    return C


def gemm_(transa, transb, alpha, A, B, beta, C, stream=None):
    """BLAS.gemm!(tA, tB, alpha, A, B, beta, C) -> C."""
    pa, ra, ca, lda = _colmajor(A, "A")
    pb, rb, cb, ldb = _colmajor(B, "B")
    pc, m, n, ldc = _colmajor(C, "C")
    k = ca if transa in ('N', 'n') else ra
    check(lib().dg_gemm(ch(transa), ch(transb), m, n, k, float(alpha), pa, lda, pb, ldb,
                        float(beta), pc, ldc, _stream(stream)))
    return C


def gemm_f64_emulated_tn(alpha, A, B, beta, C, stream=None):
    """C = alpha A'B + beta C in FP64 with the products on the BF16 tensor
    cores (A k x m, B k x n, k <= 1024): the tile update of engine 2."""
    pa, k, m, lda = _colmajor(A, "A")
    pb, kb, n, ldb = _colmajor(B, "B")
    pc, mc, nc, ldc = _colmajor(C, "C")
    if kb != k or mc != m or nc != n:
        raise ValueError("gemm_f64_emulated_tn: shapes A'%dx%d, B %dx%d, C %dx%d do not match"
                         % (m, k, kb, n, mc, nc))
    check(lib().dg_gemm_f64_emulated_tn(m, n, k, float(alpha), pa, lda, pb, ldb, float(beta), pc,
                                        ldc, _stream(stream)))
    return C


F64_ENGINES = {"dfma": 0, "dmma": 1, "emulated": 2}


def set_f64_engine(engine) -> str:
    """Selects the engine of the FP64 tile updates ("dfma", "dmma" or
    "emulated": trailing SYRK/GEMM on the tensor cores with FP64 accuracy,
    POTRF/TRSM on DFMA); returns the previous one.  Process-wide."""
    code = F64_ENGINES[engine] if isinstance(engine, str) else int(engine)
    if code not in F64_ENGINES.values():
        raise ValueError("unknown FP64 engine %r" % (engine,))
    old = lib().dg_set_f64_engine(code)
    return {v: k for k, v in F64_ENGINES.items()}[old]


def get_f64_engine() -> str:
    """The current engine of the FP64 tile updates (see set_f64_engine)."""
    return {v: k for k, v in F64_ENGINES.items()}[lib().dg_get_f64_engine()]


def trsv_(uplo, trans, diag, A, x, stream=None):
    """BLAS.trsv!(uplo, trans, diag, A, x) -> x."""
    pa, n, _, lda = _colmajor(A, "A")
    px, _, _, _ = _colmajor(x, "x")
    check(lib().dg_trsv(ch(uplo), ch(trans), ch(diag), n, pa, lda, px, _stream(stream)))
    return x


def gemv_(trans, alpha, A, x, beta, y, stream=None):
    """BLAS.gemv!(trans, alpha, A, x, beta, y) -> y."""
    pa, m, n, lda = _colmajor(A, "A")
    px, _, _, _ = _colmajor(x, "x")
    py, _, _, _ = _colmajor(y, "y")
    check(lib().dg_gemv(ch(trans), m, n, float(alpha), pa, lda, px, float(beta), py,
                        _stream(stream)))
    return y


# ---------------------------------------------------------------------------
# whole-array calls
# ---------------------------------------------------------------------------

class Cholesky:
    """LinearAlgebra.Cholesky{T,<:DMatrix}: the factor tiles and uplo.

    With the emulated FP64 engine the factorization also keeps the
    transposed inverses of its diagonal tiles (winv, formed for the panel
    products anyway), which ldiv_ applies as emulated products; a Cholesky
    built from factors alone solves by substitution.  winv_nb is the block
    size the inverses were formed at (the factorization's square blocks)."""

    def __init__(self, factors: DArray, uplo: str, info: int, winv=None, winv_nb=None):
        self.factors = factors
        self.uplo = uplo
        self.info = info
        self.winv = winv
        self.winv_nb = winv_nb

    @property
    def U(self) -> torch.Tensor:
        F = self.factors.collect()
        return torch.triu(F) if self.uplo == 'U' else torch.triu(F.T)

    @property
    def L(self) -> torch.Tensor:
        F = self.factors.collect()
        return torch.tril(F) if self.uplo == 'L' else torch.tril(F.T)

    def issuccess(self) -> bool:
        return self.info == 0


def _dims2(A: DArray):
    return (A.shape[0], A.shape[1]) if A.ndim == 2 else (A.shape[0], 1)


def _blocks2(part: Blocks):
    return part.blocksize if len(part.blocksize) == 2 else (part.blocksize[0], 1)


def copy_reblock(src: DArray, dst: DArray, stream=None) -> DArray:
    """copyto!(dst, src) between two tilings of one matrix, on the device
    (darray_copyto! of copy_buffered, src/array/copy.jl:11-37)."""
    if src.shape != dst.shape:
        raise ValueError(f"copyto!: shapes {src.shape} and {dst.shape} differ")
    m, n = _dims2(src)
    smb, snb = _blocks2(src.partitioning)
    dmb, dnb = _blocks2(dst.partitioning)
    check(lib().dg_copy_reblock(m, n, smb, snb, src.tile_ptrs(), dmb, dnb, dst.tile_ptrs(),
                                _stream(stream)))
    return dst


def _buffered(A: DArray, part: Blocks, stream=None) -> DArray:
    """The argument as the region needs it: A itself when its partitioning is
    already `part`, else a copy re-blocked to `part` (maybe_copy_buffered,
    copy.jl:3-10; allocate_copy_buffer, copy.jl:34-36)."""
    if A.partitioning == part:
        return A
    buf = DArray(A.shape, part, device=A.storage.device, dtype=A.dtype)
    return copy_reblock(A, buf, stream)


def _square_blocks(A: DArray):
    if A.ndim != 2 or A.shape[0] != A.shape[1]:
        raise ValueError(f"matrix is not square: dimensions are {A.shape}")  # checksquare
    return min(A.partitioning.blocksize)


def cholesky_(A: DArray, uplo: str = 'U', check_: bool = True, stream=None) -> Cholesky:
    """cholesky!(DA): in-place tiled factorization (_chol!, cholesky.jl:19-108).
    A DArray blocked Blocks(mb, nb) with mb != nb is factored in a copy
    re-blocked to Blocks(min, min) and copied back (maybe_copy_buffered,
    cholesky.jl:34)."""
    if uplo not in ('U', 'L'):
        raise ValueError("uplo must be 'U' or 'L'")
    nb = _square_blocks(A)
    W = _buffered(A, Blocks(nb, nb), stream)
    n = A.shape[0]
    winv = None
    if n > 0 and nb <= 1024 and lib().dg_get_f64_engine() == F64_ENGINES["emulated"]:
        mt = (n + nb - 1) // nb
        winv = torch.empty(mt * nb * nb, dtype=torch.float64, device=A.storage.device)
        rc = lib().dg_cholesky_tiled_winv(ch(uplo), n, nb, W.tile_ptrs(), winv.data_ptr(),
                                          _stream(stream))
    else:
        rc = lib().dg_cholesky_tiled(ch(uplo), n, nb, W.tile_ptrs(), _stream(stream))
    if rc < 0:
        check(rc)
    if W is not A:
        copy_reblock(W, A, stream)
    if rc > 0:
        winv = None
        if check_:
            raise PosDefException(rc)
    return Cholesky(A, uplo, rc, winv, winv_nb=nb)


def cholesky_distribute(A, part: Blocks, uplo: str = 'U', check_: bool = True, stream=None,
                        out: DArray | None = None) -> Cholesky:
    """cholesky(distribute(A, Blocks(nb, nb))) for a square array A on the host.

    The tiles move to the device inside the factorization's graph, one upload
    task per tile, so each tile's first task waits only for its own transfer
    and the transfers overlap the first steps' updates; Dagger moves a CPU
    chunk to the GPU processor when the first task that needs it runs
    (ext/CUDAExt.jl:329-348).  A: numpy array or torch tensor (host or device),
    read C-contiguous in FP64; a Cholesky's input is symmetric, so the row-major
    layout reads the same as Julia's column-major one.  A host tensor that is
    not page-locked is first copied into page-locked memory.  out: a DArray of
    A's shape and Blocks(nb, nb) to receive the tiles (allocated if None).
    Returns the Cholesky of the tiles, as cholesky_ does."""
    if uplo not in ('U', 'L'):
        raise ValueError("uplo must be 'U' or 'L'")
    t = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float64)) if isinstance(A, np.ndarray) else A
    if t.ndim != 2 or t.shape[0] != t.shape[1]:
        raise ValueError(f"matrix is not square: dimensions are {tuple(t.shape)}")
    t = t.to(torch.float64).contiguous()
    if not t.is_cuda and not t.is_pinned():
        t = t.pin_memory()
    n = t.shape[0]
    if len(part.blocksize) != 2 or part.blocksize[0] != part.blocksize[1]:
        raise ValueError("the Cholesky path needs square blocks Blocks(nb, nb)")
    nb = part.blocksize[0]
    D = out if out is not None else DArray((n, n), part,
                                           device=t.device if t.is_cuda else None)
    if D.shape != (n, n) or D.partitioning != part:
        raise ValueError("out must have A's shape and the same Blocks")
    winv = None
    if n > 0 and nb <= 1024 and lib().dg_get_f64_engine() == F64_ENGINES["emulated"]:
        mt = (n + nb - 1) // nb
        winv = torch.empty(mt * nb * nb, dtype=torch.float64, device=D.storage.device)
    rc = lib().dg_cholesky_tiled_host(ch(uplo), n, nb, t.data_ptr(), t.stride(0), D.tile_ptrs(),
                                      winv.data_ptr() if winv is not None else None,
                                      _stream(stream))
    if rc < 0:
        check(rc)
    if rc > 0:
        winv = None
        if check_:
            raise PosDefException(rc)
    return Cholesky(D, uplo, rc, winv, winv_nb=nb)


def cholesky(A: DArray, uplo: str = 'U', check_: bool = True, stream=None) -> Cholesky:
    """cholesky(DA): cholcopy (cholesky.jl:1) then cholesky!."""
    return cholesky_(A.copy(), uplo, check_, stream)


def ldiv_(C, B: DArray, stream=None) -> DArray:
    """ldiv!(C, B): B <- A^-1 B with A = U'U or LL' (linalg.jl:352-405), or
    with A = P' L U for an LU (linalg.jl:264-278).

    B is an N-vector or an N x r matrix.  As in the reference, the factor
    and B are solved at Blocks(min_bsa, min_bsa) (Blocks(min_bsa) for a
    vector), min_bsa the factor's smaller block size; an argument blocked
    otherwise is copied to that blocking and back (maybe_copy_buffered,
    linalg.jl:362-364)."""
    if isinstance(C, LU):
        return _ldiv_lu(C, B, stream)
    F = C.factors
    if B.shape[0] != F.shape[0]:
        raise ValueError("dimension mismatch")
    nb = min(F.partitioning.blocksize)
    partB = Blocks(nb) if B.ndim == 1 else Blocks(nb, nb)
    Fb = _buffered(F, Blocks(nb, nb), stream)
    Bb = _buffered(B, partB, stream)
    nrhs = 1 if B.ndim == 1 else B.shape[1]
    if (C.winv is not None and C.winv_nb == nb
            and lib().dg_get_f64_engine() == F64_ENGINES["emulated"]):
        rc = lib().dg_cholesky_solve_tiled_winv(ch(C.uplo), F.shape[0], nb, Fb.tile_ptrs(),
                                                C.winv.data_ptr(), nrhs, Bb.tile_ptrs(),
                                                _stream(stream))
    else:
        rc = lib().dg_cholesky_solve_tiled(ch(C.uplo), F.shape[0], nb, Fb.tile_ptrs(), nrhs,
                                           Bb.tile_ptrs(), _stream(stream))
    check(rc)
    if Bb is not B:
        copy_reblock(Bb, B, stream)
    return B


class LU:
    """LinearAlgebra.LU{T,DMatrix{T},DVector{Int}}: factors (L unit lower
    below the diagonal, U on and above it), ipiv (the 1-based global row
    interchanges, an int64 CUDA tensor of min(m, n) rows) and info."""

    def __init__(self, factors: DArray, ipiv: torch.Tensor, info: int):
        self.factors = factors
        self.ipiv = ipiv
        self.info = info

    @property
    def L(self) -> torch.Tensor:
        F = self.factors.collect()
        m, n = F.shape
        k = min(m, n)
        return torch.tril(F[:, :k], -1) + torch.eye(m, k, dtype=F.dtype, device=F.device)

    @property
    def U(self) -> torch.Tensor:
        F = self.factors.collect()
        k = min(F.shape)
        return torch.triu(F[:k, :])

    @property
    def p(self) -> torch.Tensor:
        """The row permutation (0-based): row t of P A is row p[t] of A."""
        m = self.factors.shape[0]
        perm = list(range(m))
        for i, g in enumerate(self.ipiv.tolist()):
            r = g - 1
            perm[i], perm[r] = perm[r], perm[i]
        return torch.tensor(perm, dtype=torch.int64)

    @property
    def P(self) -> torch.Tensor:
        m = self.factors.shape[0]
        return torch.eye(m, dtype=torch.float64)[self.p]

    def issuccess(self) -> bool:
        return self.info == 0

    def solve(self, B, stream=None):
        return ldiv(self, B, stream)


_PIVOTS = {"rowmaximum": 1, "nopivot": 0}


def _pivot_code(pivot) -> int:
    key = str(pivot).replace("()", "").replace("_", "").lower()
    if key not in _PIVOTS:
        raise ValueError("pivot must be 'RowMaximum' or 'NoPivot'")
    return _PIVOTS[key]


def chkfinite(A: DArray, stream=None) -> bool:
    """LAPACK.chkfinite(::DArray) (linalg.jl:126-148): True when every
    element is finite; ValueError (Julia's ArgumentError "matrix has Inf or
    NaN") otherwise.  One device pass over the tiles."""
    m, n = _dims2(A)
    mb, nb = _blocks2(A.partitioning)
    ok = lib().dg_chkfinite_tiled_mn(m, n, mb, nb, A.tile_ptrs(), _stream(stream))
    if ok < 0:
        check(ok)
    if not ok:
        raise ValueError("matrix has Inf or NaN")
    return True


_chkfinite = chkfinite


def lu_(A: DArray, pivot="RowMaximum", check_: bool = True, allowsingular: bool = False,
        stream=None) -> LU:
    """lu!(DA, RowMaximum()) / lu!(DA, NoPivot()) (src/array/lu.jl:306-410 /
    5-54): the tiled factorization in place.  Non-square Blocks(mb, nb) are
    re-blocked to Blocks(min, min) for the factorization and copied back
    (maybe_copy_buffered, copy.jl:3-37).  check_: chkfinite first, then
    SingularException(info) for an exactly zero pivot unless allowsingular."""
    code = _pivot_code(pivot)
    if A.ndim != 2:
        raise ValueError("lu needs a 2-D DArray")
    if check_:
        _chkfinite(A, stream)
    m, n = A.shape
    b = min(A.partitioning.blocksize)
    W = _buffered(A, Blocks(b, b), stream)
    nb = b
    ipiv = torch.empty(max(min(m, n), 1), dtype=torch.int64, device=A.storage.device)
    rc = lib().dg_lu_tiled(m, n, nb, W.tile_ptrs(), code, ipiv.data_ptr(), _stream(stream))
    if rc < 0:
        check(rc)
    if W is not A:
        copy_reblock(W, A, stream)
    info = rc
    if check_ and info > 0 and not allowsingular:
        raise _lib.SingularException(info)
    return LU(A if W is A else W, ipiv[:min(m, n)], info)


def lu(A: DArray, pivot="RowMaximum", check_: bool = True, allowsingular: bool = False,
       stream=None) -> LU:
    """lu(DA, pivot): _lucopy then lu! (lu.jl:1-3, 306-309)."""
    return lu_(A.copy(), pivot, check_, allowsingular, stream)


def _ldiv_lu(F: LU, B: DArray, stream=None) -> DArray:
    """ldiv!(F::LU, B) (linalg.jl:247-251): the row interchanges, then the
    unit-lower and upper block solves.  The factors and B are solved at
    Blocks(nb, nb) (Blocks(nb) for a vector), nb the factors' smaller block
    size; an argument blocked otherwise is copied there and back
    (maybe_copy_buffered, linalg.jl:262-276)."""
    A = F.factors
    n = A.shape[0]
    if A.shape[0] != A.shape[1]:
        raise ValueError("ldiv! needs a square LU")
    if B.shape[0] != n:
        raise ValueError("arguments must have the same number of rows")
    nb = min(A.partitioning.blocksize)
    Ab = _buffered(A, Blocks(nb, nb), stream)
    Bb = _buffered(B, Blocks(nb) if B.ndim == 1 else Blocks(nb, nb), stream)
    nrhs = 1 if B.ndim == 1 else B.shape[1]
    rc = lib().dg_lu_solve_tiled(n, nb, Ab.tile_ptrs(), F.ipiv.data_ptr(), nrhs, Bb.tile_ptrs(),
                                 _stream(stream))
    check(rc)
    if Bb is not B:
        copy_reblock(Bb, B, stream)
    return B


def ldiv(F: LU, B, stream=None) -> DArray:
    """ldiv(F::LU, B) / F \\ B (linalg.jl:221-262): B (a DArray, torch tensor
    or numpy array, vector or matrix) staged into a DArray blocked like the
    factors, solved in place there and returned."""
    nb = F.factors.partitioning.blocksize[0]
    src = B.collect() if isinstance(B, DArray) else B
    t = torch.as_tensor(np.asarray(src)) if isinstance(src, np.ndarray) else src
    part = Blocks(nb) if t.ndim == 1 else Blocks(nb, nb)
    BB = DArray.from_array(t.to(torch.float64), part, device=F.factors.storage.device)
    return _ldiv_lu(F, BB, stream)


def _mul_blocks(*arrays):
    """The one square block size the tile products run at: the operands'
    own when they all share Blocks(nb, nb), else the smallest block size of
    any operand (the reference's _repartition_matmatmul falls back to the
    smallest blocking, mul.jl:44-94)."""
    for X in arrays:
        if X.ndim != 2 or len(X.partitioning.blocksize) != 2:
            raise ValueError("mul needs 2-D DArrays")
    return min(min(X.partitioning.blocksize) for X in arrays)


def _buffered_all(nb, arrays, stream):
    seen = {}
    out = []
    for X in arrays:  # an operand passed twice (A === B) is copied once
        if id(X) not in seen:
            seen[id(X)] = _buffered(X, Blocks(nb, nb), stream)
        out.append(seen[id(X)])
    return out


def _trans(t: str) -> bytes:
    if t not in ('N', 'T', 'C'):
        raise ValueError(f"transpose flag must be 'N', 'T' or 'C', got {t!r}")
    return b'N' if t == 'N' else b'T'


def gemm_dagger_(C: DArray, transA: str, transB: str, A: DArray, B: DArray, alpha=1.0,
                 beta=0.0, stream=None) -> DArray:
    """gemm_dagger!(C, transA, transB, A, B, alpha, beta) (src/array/mul.jl:133-215):
    C = alpha op(A) op(B) + beta C over the tiles, one cached graph."""
    nb = _mul_blocks(A, B, C)
    m, k = (A.shape if transA == 'N' else A.shape[::-1])
    k2, n = (B.shape if transB == 'N' else B.shape[::-1])
    if k != k2 or C.shape != (m, n):
        raise ValueError(f"DimensionMismatch: op(A) {m}x{k}, op(B) {k2}x{n}, C {C.shape}")
    Ab, Bb, Cb = _buffered_all(nb, (A, B, C), stream)
    check(lib().dg_gemm_tiled(_trans(transA), _trans(transB), m, n, k, nb, float(alpha),
                              Ab.tile_ptrs(), Bb.tile_ptrs(), float(beta), Cb.tile_ptrs(),
                              _stream(stream)))
    if Cb is not C:
        copy_reblock(Cb, C, stream)
    return C


def syrk_dagger_(C: DArray, trans: str, A: DArray, alpha=1.0, beta=0.0, stream=None) -> DArray:
    """syrk_dagger!(C, trans, A, alpha, beta) (src/array/mul.jl:230-365):
    C = alpha op(A) op(A)' + beta C; the upper tiles are computed and copied
    to the lower ones (copytri!, mul.jl:368-425), so C is fully symmetric."""
    nb = _mul_blocks(A, C)
    n, k = (A.shape if trans == 'N' else A.shape[::-1])
    if C.shape != (n, n):
        raise ValueError(f"DimensionMismatch: op(A) {n}x{k}, C {C.shape}")
    Ab, Cb = _buffered_all(nb, (A, C), stream)
    check(lib().dg_syrk_tiled(_trans(trans), n, k, nb, float(alpha), Ab.tile_ptrs(), float(beta),
                              Cb.tile_ptrs(), _stream(stream)))
    if Cb is not C:
        copy_reblock(Cb, C, stream)
    return C


def mul_(C: DArray, A: DArray, B: DArray, alpha=1.0, beta=0.0, transA: str = 'N',
         transB: str = 'N', stream=None) -> DArray:
    """mul!(C, op(A), op(B), alpha, beta) on DArrays (generic_matmatmul!,
    src/array/mul.jl:11-41): A is B with exactly one of them transposed takes
    syrk_dagger!, everything else gemm_dagger!."""
    if A is B and (transA == 'N') != (transB == 'N'):
        return syrk_dagger_(C, transA if transA == 'N' else 'T', A, alpha, beta, stream)
    return gemm_dagger_(C, transA, transB, A, B, alpha, beta, stream)


def matmul(A: DArray, B: DArray, transA: str = 'N', transB: str = 'N', stream=None) -> DArray:
    """op(A) * op(B) as a new DArray with the operands' Blocks (A * B, A' * A, ...)."""
    m = A.shape[0] if transA == 'N' else A.shape[1]
    n = B.shape[1] if transB == 'N' else B.shape[0]
    C = DArray((m, n), A.partitioning, device=A.storage.device)
    return mul_(C, A, B, 1.0, 0.0, transA, transB, stream)


def ishermitian(A: DArray, stream=None) -> bool:
    """ishermitian(::DArray) (linalg.jl:90-124): diagonal tiles exactly
    symmetric; off-diagonal pairs within sqrt(eps) in Frobenius norm.  A
    DArray with Blocks(mb, nb), mb != nb, is checked on a copy re-blocked to
    Blocks(min, min), as the reference does."""
    if A.ndim != 2 or A.shape[0] != A.shape[1]:
        return False
    nb = _square_blocks(A)
    W = _buffered(A, Blocks(nb, nb), stream)
    rc = lib().dg_ishermitian_tiled(A.shape[0], nb, W.tile_ptrs(), _stream(stream))
    if rc < 0:
        check(rc)
    return rc == 1


issymmetric = ishermitian  # real FP64: the two checks coincide (linalg.jl:55-89)
