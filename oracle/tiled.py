"""CPU oracle: a restatement of Dagger.jl's tiled Cholesky factor-and-solve.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path (the `dagger_gb300`
package or `libdaggergb300.so`) imports, calls or links this module.  It is the
checker that the CUDA path is compared against, and the CPU baseline that
`bench.py` times beside the GPU.

Every function below restates one function of the reference, with the same
tile loop order, the same BLAS/LAPACK tile calls and the same alpha/beta
constants.  Tile kernels are the system LAPACK/BLAS reached through scipy
(scipy-openblas), which is what the reference's CPU path calls through
Julia's LinearAlgebra (OpenBLAS via libblastrampoline).

Reference files (paths within JuliaParallel/Dagger.jl v0.22.0):
  src/array/cholesky.jl:1-108   cholcopy, potrf_checked!, _chol! 'U' and 'L'
  src/array/trsm.jl:1-57        trsv!  (vector right-hand side)
  src/array/trsm.jl:59-192      trsm!  (matrix right-hand side)
  src/array/linalg.jl:43-54     is_cross_hermitian / is_cross_symmetric
  src/array/linalg.jl:90-124    ishermitian(::DArray)
  src/array/linalg.jl:352-405   ldiv!(::Cholesky{T,<:DMatrix}, B)
  src/array/darray.jl:107-117   Blocks partitioning (ragged last block)
  src/array/mul.jl:133-425      gemm_dagger!, syrk_dagger!, copytri!

Tiles are views into one column-major (Fortran-order) matrix: tile (i, j)
covers rows i*nb : min((i+1)*nb, m) and columns j*nb : min((j+1)*nb, n),
exactly the chunk domains a DArray with Blocks(nb, nb) has.

Parity pins: the reference publishes no golden vectors, and Julia is not
available to run it.  The oracle is pinned against FP64 LAPACK (dpotrf /
dpotrs through scipy) using the reference's own test recipes and tolerances
(test/array/linalg/cholesky.jl, test/array/linalg/solve.jl,
test/datadeps.jl:946-984, test/mpi_cholesky.jl); see tests/test_oracle.py.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import blas, lapack


# --------------------------------------------------------------------------
# partitioning (src/array/darray.jl:107-117, src/array/alloc.jl:30)
# --------------------------------------------------------------------------

def block_ranges(n: int, nb: int):
    """Index ranges of Blocks(nb) over 0..n: full blocks then one ragged block."""
    return [(s, min(s + nb, n)) for s in range(0, n, nb)] if n > 0 else []


class TileView:
    """Tile (i, j) of a Fortran-ordered matrix, as a DArray chunk."""

    def __init__(self, M: np.ndarray, nb_r: int, nb_c: int):
        assert M.flags.f_contiguous or M.ndim == 1
        self.M = M
        self.rows = block_ranges(M.shape[0], nb_r)
        self.cols = block_ranges(M.shape[1], nb_c) if M.ndim == 2 else [(0, 1)]

    @property
    def mt(self):
        return len(self.rows)

    @property
    def nt(self):
        return len(self.cols)

    def get(self, i, j):
        r0, r1 = self.rows[i]
        c0, c1 = self.cols[j]
        return self.M[r0:r1, c0:c1]

    def set(self, i, j, val):
        r0, r1 = self.rows[i]
        c0, c1 = self.cols[j]
        self.M[r0:r1, c0:c1] = val


# --------------------------------------------------------------------------
# tile kernels: the LAPACK/BLAS calls the reference makes on each tile
# --------------------------------------------------------------------------

def _potrf(uplo, a):
    """LAPACK.potrf!(uplo, A) -> (A, info); other triangle untouched."""
    c, info = lapack.dpotrf(a, lower=(uplo == 'L'), clean=0)
    return c, int(info)


def _trsm(side, uplo, trans, diag, alpha, a, b):
    """BLAS.trsm!(side, uplo, transa, diag, alpha, A, B) -> B."""
    if b.size == 0:
        return b.copy()
    return blas.dtrsm(alpha, a, b, side=(side == 'R'), lower=(uplo == 'L'),
                      trans_a=(trans != 'N'), diag=(diag == 'U'))


def _syrk(uplo, trans, alpha, a, beta, c):
    """BLAS.syrk!(uplo, trans, alpha, A, beta, C) -> C (one triangle)."""
    return blas.dsyrk(alpha, a, beta=beta, c=c, trans=(trans != 'N'),
                      lower=(uplo == 'L'))


def _gemm(ta, tb, alpha, a, b, beta, c):
    """BLAS.gemm!(tA, tB, alpha, A, B, beta, C) -> C."""
    if c.size == 0:
        return c.copy()
    return blas.dgemm(alpha, a, b, beta=beta, c=c, trans_a=(ta != 'N'),
                      trans_b=(tb != 'N'))


def _trsv(uplo, trans, diag, a, x):
    """BLAS.trsv!(uplo, trans, diag, A, x) -> x."""
    return blas.dtrsv(a, x, lower=(uplo == 'L'), trans=(0 if trans == 'N' else 1),
                      diag=(diag == 'U'))


def _gemv(trans, alpha, a, x, beta, y):
    """BLAS.gemv!(trans, alpha, A, x, beta, y) -> y."""
    return blas.dgemv(alpha, a, x, beta=beta, y=y, trans=(0 if trans == 'N' else 1))


class PosDefException(Exception):
    """LinearAlgebra.PosDefException(info)."""

    def __init__(self, info):
        super().__init__(f"matrix is not positive definite; Cholesky factorization failed (info={info})")
        self.info = info


# --------------------------------------------------------------------------
# factorization (src/array/cholesky.jl)
# --------------------------------------------------------------------------

def chol_tiled(A: np.ndarray, nb: int, uplo: str = 'U'):
    """_chol!(A, UpperTriangular|LowerTriangular) on a Fortran-ordered copy of A.

    Follows src/array/cholesky.jl:19-63 ('U') and :64-108 ('L'): the
    right-looking tile loop POTRF(k,k); TRSM of the row ('U') or column ('L')
    panel; SYRK on the diagonal trailing tiles; GEMM on the off-diagonal
    trailing tiles, in the order the reference spawns them.  Tasks run
    sequentially in submission order, which the datadeps rules make
    equivalent to the parallel schedule (src/datadeps/queue.jl:50-53).

    Returns (F, info).  info is the LAPACK convention for the whole matrix:
    0 on success, else the 1-based order of the leading minor that is not
    positive definite.  potrf_checked! (cholesky.jl:2-18) stops the region at
    the first failing POTRF; the tiles after it keep their partially updated
    values.  (The reference records the tile-local LAPACK info and its
    PosDefException test is marked broken, test/array/linalg/cholesky.jl:47;
    the global order is what LinearAlgebra's dense cholesky reports.)
    """
    assert uplo in ('U', 'L')
    n = A.shape[0]
    assert A.shape == (n, n)
    F = np.array(A, dtype=np.float64, order='F', copy=True)
    T = TileView(F, nb, nb)
    mt = nt = T.mt
    for k in range(mt):
        akk, info = _potrf(uplo, T.get(k, k))
        T.set(k, k, akk)
        if info != 0:
            return F, T.rows[k][0] + info
        if uplo == 'U':
            for j in range(k + 1, nt):                          # cholesky.jl:40-42
                T.set(k, j, _trsm('L', 'U', 'T', 'N', 1.0, T.get(k, k), T.get(k, j)))
            for m in range(k + 1, mt):                          # cholesky.jl:43-52
                T.set(m, m, _syrk('U', 'T', -1.0, T.get(k, m), 1.0, T.get(m, m)))
                for j in range(m + 1, nt):
                    T.set(m, j, _gemm('T', 'N', -1.0, T.get(k, m), T.get(k, j), 1.0, T.get(m, j)))
        else:
            for m in range(k + 1, mt):                          # cholesky.jl:85-87
                T.set(m, k, _trsm('R', 'L', 'T', 'N', 1.0, T.get(k, k), T.get(m, k)))
            for j in range(k + 1, nt):                          # cholesky.jl:88-97
                T.set(j, j, _syrk('L', 'N', -1.0, T.get(j, k), 1.0, T.get(j, j)))
                for m in range(j + 1, mt):
                    T.set(m, j, _gemm('N', 'T', -1.0, T.get(m, k), T.get(j, k), 1.0, T.get(m, j)))
    return F, 0


def cholesky(A: np.ndarray, nb: int, uplo: str = 'U'):
    """cholesky(DA): cholcopy (cholesky.jl:1) then the tiled factor; raises on failure."""
    F, info = chol_tiled(A, nb, uplo)
    if info != 0:
        raise PosDefException(info)
    return F


def chol_tasks(mt: int, uplo: str = 'U'):
    """The task list _chol! spawns, in submission order, with In/InOut tiles.

    Each entry is (kind, reads, writes) with tiles as (i, j) pairs; this is
    the DAG that datadeps sees (cholesky.jl:38-53 and :83-98).
    """
    tasks = []
    for k in range(mt):
        tasks.append(('potrf', [], [(k, k)]))
        if uplo == 'U':
            for j in range(k + 1, mt):
                tasks.append(('trsm', [(k, k)], [(k, j)]))
            for m in range(k + 1, mt):
                tasks.append(('syrk', [(k, m)], [(m, m)]))
                for j in range(m + 1, mt):
                    tasks.append(('gemm', [(k, m), (k, j)], [(m, j)]))
        else:
            for m in range(k + 1, mt):
                tasks.append(('trsm', [(k, k)], [(m, k)]))
            for j in range(k + 1, mt):
                tasks.append(('syrk', [(j, k)], [(j, j)]))
                for m in range(j + 1, mt):
                    tasks.append(('gemm', [(m, k), (j, k)], [(m, j)]))
    return tasks


def datadeps_edges(tasks):
    """Dependency edges by the datadeps rules (src/datadeps/queue.jl:43-53,
    src/datadeps/aliasing.jl:740-776): a writer waits for the last writer and
    every reader since; a reader waits for the last writer.  Tiles alias only
    themselves.  Returns a list of predecessor sets, one per task."""
    last_writer = {}
    readers = {}
    preds = []
    for t, (_, reads, writes) in enumerate(tasks):
        p = set()
        for tile in reads:
            if tile in last_writer:
                p.add(last_writer[tile])
        for tile in writes:
            if tile in last_writer:
                p.add(last_writer[tile])
            p.update(readers.get(tile, ()))
        for tile in reads:
            readers.setdefault(tile, []).append(t)
        for tile in writes:
            last_writer[tile] = t
            readers[tile] = []
        p.discard(t)
        preds.append(p)
    return preds


# --------------------------------------------------------------------------
# triangular solves (src/array/trsm.jl)
# --------------------------------------------------------------------------

def trsm_tiled(side, uplo, trans, diag, alpha, A: np.ndarray, B: np.ndarray, nb: int):
    """Dagger.trsm!(side, uplo, trans, diag, alpha, A, B) (trsm.jl:59-192).

    A is N x N tiled Blocks(nb, nb); B is tiled Blocks(nb, nb) too
    (ldiv! re-blocks B to the factor's block size, linalg.jl:364).  Loop
    orders, the lalpha rule (alpha on the first step, 1 afterwards, passed as
    the GEMM beta) and tile index reversals are the reference's.  B is
    updated in place and returned.
    """
    TA = TileView(A, nb, nb)
    TB = TileView(B, nb, nb)
    Bmt, Bnt = TB.mt, TB.nt
    one, mone = 1.0, -1.0
    a, b = TA.get, TB.get
    if side == 'L':
        if uplo == 'U' and trans == 'N':                        # trsm.jl:91-102
            for k in range(1, Bmt + 1):
                la = alpha if k == 1 else one
                kk = Bmt - k
                for n in range(Bnt):
                    TB.set(kk, n, _trsm(side, uplo, trans, diag, la, a(kk, kk), b(kk, n)))
                for m in range(k + 1, Bmt + 1):
                    mm = Bmt - m
                    for n in range(Bnt):
                        TB.set(mm, n, _gemm('N', 'N', mone, a(mm, kk), b(kk, n), la, b(mm, n)))
        elif uplo == 'U':                                       # trsm.jl:103-114
            for k in range(Bmt):
                la = alpha if k == 0 else one
                for n in range(Bnt):
                    TB.set(k, n, _trsm(side, uplo, trans, diag, la, a(k, k), b(k, n)))
                for m in range(k + 1, Bmt):
                    for n in range(Bnt):
                        TB.set(m, n, _gemm(trans, 'N', mone, a(k, m), b(k, n), la, b(m, n)))
        elif trans == 'N':                                      # trsm.jl:117-128 ('L','L','N')
            for k in range(Bmt):
                la = alpha if k == 0 else one
                for n in range(Bnt):
                    TB.set(k, n, _trsm(side, uplo, trans, diag, la, a(k, k), b(k, n)))
                for m in range(k + 1, Bmt):
                    for n in range(Bnt):
                        TB.set(m, n, _gemm('N', 'N', mone, a(m, k), b(k, n), la, b(m, n)))
        else:                                                   # trsm.jl:129-140 ('L','L','T')
            for k in range(1, Bmt + 1):
                la = alpha if k == 1 else one
                kk = Bmt - k
                for n in range(Bnt):
                    TB.set(kk, n, _trsm(side, uplo, trans, diag, la, a(kk, kk), b(kk, n)))
                for m in range(k + 1, Bmt + 1):
                    mm = Bmt - m
                    for n in range(Bnt):
                        TB.set(mm, n, _gemm(trans, 'N', mone, a(kk, mm), b(kk, n), la, b(mm, n)))
    else:
        if uplo == 'U' and trans == 'N':                        # trsm.jl:145-156
            for k in range(Bnt):
                la = alpha if k == 0 else one
                for m in range(Bmt):
                    TB.set(m, k, _trsm(side, uplo, trans, diag, la, a(k, k), b(m, k)))
                for m in range(Bmt):
                    for n in range(k + 1, Bnt):
                        TB.set(m, n, _gemm('N', 'N', mone, b(m, k), a(k, n), la, b(m, n)))
        elif uplo == 'U':                                       # trsm.jl:157-165
            for k in range(1, Bnt + 1):
                kk = Bnt - k
                for m in range(Bmt):
                    TB.set(m, kk, _trsm(side, uplo, trans, diag, alpha, a(kk, kk), b(m, kk)))
                    for n in range(k + 1, Bnt + 1):
                        nn = Bnt - n
                        TB.set(m, nn, _gemm('N', trans, mone, b(m, kk), a(nn, kk), one, b(m, nn)))
        elif trans == 'N':                                      # trsm.jl:168-176
            for k in range(1, Bnt + 1):
                la = alpha if k == 1 else one
                kk = Bnt - k
                for m in range(Bmt):
                    TB.set(m, kk, _trsm(side, uplo, trans, diag, la, a(kk, kk), b(m, kk)))
                    for n in range(k + 1, Bnt + 1):
                        nn = Bnt - n
                        TB.set(m, nn, _gemm('N', 'N', mone, b(m, kk), a(kk, nn), la, b(m, nn)))
        else:                                                   # trsm.jl:178-186
            for k in range(Bnt):
                for m in range(Bmt):
                    TB.set(m, k, _trsm(side, uplo, trans, diag, alpha, a(k, k), b(m, k)))
                    for n in range(k + 1, Bnt):
                        TB.set(m, n, _gemm('N', trans, mone, b(m, k), a(n, k), one, b(m, n)))
    return B


def trsv_tiled(uplo, trans, diag, alpha, A: np.ndarray, x: np.ndarray, nb: int):
    """Dagger.trsv!(uplo, trans, diag, alpha, A, b) (trsm.jl:1-57), in place.

    Restated as the reference writes it: TRSV on the diagonal tile (BLAS
    trsv has no alpha), then GEMV updates of the other blocks with
    beta = lalpha.  Its only caller, ldiv!, passes alpha = 1.
    """
    n = A.shape[0]
    r = block_ranges(n, nb)
    TA = TileView(A, nb, nb)
    Bnt = len(r)
    one, mone = 1.0, -1.0

    def xs(i):
        return x[r[i][0]:r[i][1]]

    def setx(i, v):
        x[r[i][0]:r[i][1]] = v

    if uplo == 'U':
        if trans == 'N':                                        # trsm.jl:18-25
            for k in reversed(range(Bnt)):
                la = alpha if k == Bnt - 1 else one
                setx(k, _trsv('U', 'N', diag, TA.get(k, k), xs(k)))
                for i in range(k):
                    setx(i, _gemv('N', mone, TA.get(i, k), xs(k), la, xs(i)))
        else:                                                   # trsm.jl:26-33
            for k in range(Bnt):
                la = alpha if k == 0 else one
                setx(k, _trsv('U', trans, diag, TA.get(k, k), xs(k)))
                for i in range(k + 1, Bnt):
                    setx(i, _gemv(trans, mone, TA.get(k, i), xs(k), la, xs(i)))
    else:
        if trans == 'N':                                        # trsm.jl:36-43
            for k in range(Bnt):
                la = alpha if k == 0 else one
                setx(k, _trsv('L', 'N', diag, TA.get(k, k), xs(k)))
                for i in range(k + 1, Bnt):
                    setx(i, _gemv('N', mone, TA.get(i, k), xs(k), la, xs(i)))
        else:                                                   # trsm.jl:44-51
            for k in reversed(range(Bnt)):
                la = alpha if k == Bnt - 1 else one
                setx(k, _trsv('L', trans, diag, TA.get(k, k), xs(k)))
                for i in range(k):
                    setx(i, _gemv(trans, mone, TA.get(k, i), xs(k), la, xs(i)))
    return x


def ldiv_cholesky(F: np.ndarray, uplo: str, B: np.ndarray, nb: int):
    """ldiv!(C::Cholesky{T,<:DMatrix}, B) (linalg.jl:352-405), in place on B.

    'U': solve U' y = B (trsm 'L','U','T'), then U x = y (trsm 'L','U','N').
    'L': solve L y = B (trsm 'L','L','N'), then L' x = y (trsm 'L','L','T').
    A vector B goes through trsv! with the same order (linalg.jl:366-383).
    """
    if B.ndim == 1:
        if uplo == 'U':
            trsv_tiled('U', 'T', 'N', 1.0, F, B, nb)
            trsv_tiled('U', 'N', 'N', 1.0, F, B, nb)
        else:
            trsv_tiled('L', 'N', 'N', 1.0, F, B, nb)
            trsv_tiled('L', 'T', 'N', 1.0, F, B, nb)
        return B
    assert B.flags.f_contiguous
    if uplo == 'U':
        trsm_tiled('L', 'U', 'T', 'N', 1.0, F, B, nb)
        trsm_tiled('L', 'U', 'N', 'N', 1.0, F, B, nb)
    else:
        trsm_tiled('L', 'L', 'N', 'N', 1.0, F, B, nb)
        trsm_tiled('L', 'L', 'T', 'N', 1.0, F, B, nb)
    return B


# --------------------------------------------------------------------------
# symmetry check (src/array/linalg.jl:43-54, 90-124)
# --------------------------------------------------------------------------

def ishermitian_tiled(A: np.ndarray, nb: int) -> bool:
    """ishermitian(::DArray): diagonal tiles must be exactly symmetric
    (Base ishermitian on the chunk); off-diagonal pairs pass when
    ||A_ij - A_ji'||_F <= sqrt(eps) * max(||A_ij||_F, ||A_ji||_F)."""
    n, m = A.shape
    if n != m:
        return False
    T = TileView(np.asfortranarray(A), nb, nb)
    rtol = np.sqrt(np.finfo(np.float64).eps)
    for i in range(T.mt):
        d = T.get(i, i)
        if not np.array_equal(d, d.T):
            return False
    for i in range(1, T.mt):
        for j in range(i):
            a1, a2 = T.get(i, j), T.get(j, i).T
            if np.linalg.norm(a1 - a2) > rtol * max(np.linalg.norm(a1), np.linalg.norm(a2)):
                return False
    return True


# --------------------------------------------------------------------------
# DArray multiplication (src/array/mul.jl)
# --------------------------------------------------------------------------

def gemm_dagger(C: np.ndarray, transA: str, transB: str, A: np.ndarray, B: np.ndarray,
                alpha: float, beta: float, nb: int) -> np.ndarray:
    """gemm_dagger! (mul.jl:133-215): for every C tile (m, n), the k loop of
    gemm!(transA, transB, alpha, op(A) tile, op(B) tile, k == 1 ? beta : 1)."""
    Cf = np.asfortranarray(C.copy())
    TA = TileView(np.asfortranarray(A), nb, nb)
    TB = TileView(np.asfortranarray(B), nb, nb)
    TC = TileView(Cf, nb, nb)
    kt = TA.nt if transA == 'N' else TA.mt
    for m in range(TC.mt):
        for n in range(TC.nt):
            for k in range(kt):
                a = TA.get(m, k) if transA == 'N' else TA.get(k, m)
                b = TB.get(k, n) if transB == 'N' else TB.get(n, k)
                TC.set(m, n, _gemm(transA, transB, alpha, a, b, beta if k == 0 else 1.0,
                                   np.asfortranarray(TC.get(m, n))))
    return Cf


def syrk_dagger(C: np.ndarray, trans: str, A: np.ndarray, alpha: float, beta: float,
                nb: int) -> np.ndarray:
    """syrk_dagger! (mul.jl:230-365) with uplo = 'U', then copytri! (mul.jl:368-425):
    syrk! on the diagonal tiles and gemm! above them, each with beta on its
    first term, then the upper tiles transposed into the lower ones."""
    Cf = np.asfortranarray(C.copy())
    TA = TileView(np.asfortranarray(A), nb, nb)
    TC = TileView(Cf, nb, nb)
    kt = TA.nt if trans == 'N' else TA.mt
    tile = (lambda i, k: TA.get(i, k)) if trans == 'N' else (lambda i, k: TA.get(k, i))
    other = 'T' if trans == 'N' else 'N'
    for n in range(TC.nt):
        for k in range(kt):
            TC.set(n, n, _syrk('U', trans, alpha, tile(n, k), beta if k == 0 else 1.0,
                               np.asfortranarray(TC.get(n, n))))
        for m in range(n + 1, TC.mt):
            for k in range(kt):
                ta, tb = (trans, other)
                TC.set(n, m, _gemm(ta, tb, alpha, tile(n, k), tile(m, k), beta if k == 0 else 1.0,
                                   np.asfortranarray(TC.get(n, m))))
    for i in range(TC.mt):  # copytri!(C, 'U')
        for j in range(i, TC.mt):
            if i == j:
                d = TC.get(i, i)
                TC.set(i, i, np.triu(d) + np.triu(d, 1).T)
            else:
                TC.set(j, i, TC.get(i, j).T)
    return Cf


# --------------------------------------------------------------------------
# accuracy measures reported for every result
# --------------------------------------------------------------------------

def triangle(F: np.ndarray, uplo: str) -> np.ndarray:
    return np.triu(F) if uplo == 'U' else np.tril(F)


def factor_residual(A: np.ndarray, F: np.ndarray, uplo: str) -> float:
    """||A - U'U||_F / ||A||_F (or ||A - LL'||_F / ||A||_F)."""
    T = triangle(F, uplo)
    R = T.T @ T if uplo == 'U' else T @ T.T
    return float(np.linalg.norm(A - R) / np.linalg.norm(A))


def backward_error(A: np.ndarray, X: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Normwise backward error per right-hand side, infinity norms:
    ||b - A x|| / (||A|| ||x|| + ||b||)."""
    X2 = X.reshape(X.shape[0], -1)
    B2 = B.reshape(B.shape[0], -1)
    R = B2 - A @ X2
    nA = np.abs(A).sum(axis=1).max()
    return np.abs(R).max(axis=0) / (nA * np.abs(X2).max(axis=0) + np.abs(B2).max(axis=0))


def lapack_factor(A: np.ndarray, uplo: str = 'U'):
    """Untiled FP64 LAPACK dpotrf: the FP64 LAPACK reference factor."""
    c, info = lapack.dpotrf(np.asfortranarray(A), lower=(uplo == 'L'), clean=1)
    return c, int(info)


def lapack_solve(A: np.ndarray, B: np.ndarray, uplo: str = 'U'):
    c, info = lapack_factor(A, uplo)
    assert info == 0
    x, info = lapack.dpotrs(c, B, lower=(uplo == 'L'))
    assert info == 0
    return x


# --------------------------------------------------------------------------
# seeded input generators for the benchmark configurations
# --------------------------------------------------------------------------

def spd_uniform(n: int, seed: int) -> np.ndarray:
    """A = B B' / n + n I with B i.i.d. uniform[-1, 1] (numpy PCG64(seed))."""
    rng = np.random.Generator(np.random.PCG64(seed))
    B = rng.uniform(-1.0, 1.0, size=(n, n))
    A = B @ B.T / n
    A[np.diag_indices(n)] += n
    return np.asfortranarray(A)


def spd_spectrum(n: int, cond: float, seed: int) -> np.ndarray:
    """A = Q diag(l) Q' with Q from QR of a seeded Gaussian, l log-spaced on [1, cond]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    G = rng.standard_normal((n, n))
    Q, _ = np.linalg.qr(G)
    lam = np.logspace(0.0, np.log10(cond), n)
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    return np.asfortranarray(A)


def rhs_normal(n: int, nrhs: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed + 1_000_003))
    return np.asfortranarray(rng.standard_normal((n, nrhs)))
