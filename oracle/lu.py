"""CPU oracle: a restatement of Dagger.jl's tiled LU factorization and solve.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path (the `dagger_gb300`
package or `libdaggergb300.so`) imports, calls or links this module.  It is the
checker that the CUDA path is compared against, and the CPU baseline that
`bench.py` times beside the GPU for the LU row.

Reference files (paths within JuliaParallel/Dagger.jl v0.22.0):
  src/array/lu.jl:5-54      lu!(A, NoPivot()): generic_lufact! on the diagonal
                            tile, TRSM('R','U','N','N') of the column panel,
                            TRSM('L','L','N','U') of the row panel, GEMM('N','N')
  src/array/lu.jl:129-185   swaprows_trail!: a panel's interchanges between tile
                            (k, j) and tile (i, j), in pivot order
  src/array/lu.jl:263-304   factor_panel_lapack!: the block column from the
                            diagonal down factored by one LAPACK getrf
  src/array/lu.jl:306-410   lu!(A, RowMaximum()): panel, interchanges in every
                            other block column, TRSM, GEMM
  src/array/linalg.jl:264-308  ldiv!(F::LU, B): _apply_ipiv_rows! (one
                            swaprows_trail! per tile pair), then
                            ldiv!(UnitLowerTriangular) and ldiv!(UpperTriangular)
                            as Dagger.trsm! (trsm.jl:59-192)

Tile kernels are LAPACK/BLAS through scipy (getrf, trsm, gemm), the calls the
reference's CPU path makes through Julia's LinearAlgebra.  generic_lufact!
(Julia's LinearAlgebra, generic LU without pivoting) is restated below from
its published algorithm: for each column, multipliers scaled by the inverse
of the pivot (skipped, with info set, when the pivot is zero), then the
rank-1 update of the trailing block.

Parity pins: the reference publishes no golden vectors.  The pivoted oracle is
pinned against untiled LAPACK dgetrf (same pivots, same factors to rounding)
and the reference's own test recipes (test/array/linalg/lu.jl: P A = L U to
rtol 1e-12 pivoted / 1e-7 unpivoted, the solve against A \\ b to 1e-6,
SingularException for ones(128, 128)); see tests/test_oracle_lu.py.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

from .tiled import TileView, _gemm, _trsm, trsm_tiled, trsv_tiled


class SingularException(Exception):
    """LinearAlgebra.SingularException(info)."""

    def __init__(self, info):
        super().__init__(f"SingularException({info})")
        self.info = info


def generic_lufact_nopivot(a: np.ndarray):
    """generic_lufact!(A, NoPivot()) on one tile -> (A, info): for k, the
    column below the diagonal times inv(A[k, k]) (when A[k, k] != 0, else
    info = k), then A[k+1:, k+1:] -= A[k+1:, k] A[k, k+1:]."""
    a = np.array(a, dtype=np.float64, order='F', copy=True)
    m, n = a.shape
    info = 0
    for k in range(min(m, n)):
        if a[k, k] != 0.0:
            a[k + 1:, k] *= 1.0 / a[k, k]
        elif info == 0:
            info = k + 1
        a[k + 1:, k + 1:] -= np.outer(a[k + 1:, k], a[k, k + 1:])
    return a, info


def _getrf(a: np.ndarray):
    """LAPACK.getrf!(A) -> (A, ipiv 1-based, info)."""
    lu, piv, info = lapack.dgetrf(np.asfortranarray(a), overwrite_a=0)
    return lu, piv.astype(np.int64) + 1, int(info)


def swaprows_trail(A: np.ndarray, M: np.ndarray, ipiv_k: np.ndarray, i: int, mb: int):
    """swaprows_trail!(A, M, ipiv, m, mb) (lu.jl:129-185), 0-based block index
    i: for every pivot p of the chunk (in order) whose global row lies in
    block i, row p of A trades places with that row of M."""
    for p, g in enumerate(ipiv_k):
        q, r = divmod(int(g) - 1, mb)
        if q == i:
            tmp = A[p, ...].copy()
            A[p, ...] = M[r, ...]
            M[r, ...] = tmp


def lu_rowmaximum(A: np.ndarray, nb: int):
    """lu!(A, RowMaximum()) with the LAPACK panel (lu.jl:306-410 with
    factor_panel_lapack!).  Returns (factors, ipiv 1-based global, info)."""
    F = np.array(A, dtype=np.float64, order='F', copy=True)
    m, n = F.shape
    T = TileView(F, nb, nb)
    mt, nt = T.mt, T.nt
    ipiv = np.arange(1, min(m, n) + 1, dtype=np.int64)
    info = 0
    for k in range(min(mt, nt)):
        r0 = T.rows[k][0]
        c0, c1 = T.cols[k]
        panel = F[r0:, c0:c1]                                    # factor_panel_lapack!
        lu, piv, linfo = _getrf(panel)
        F[r0:, c0:c1] = lu
        if info == 0 and linfo != 0:
            info = r0 + linfo
        npiv = len(piv)
        ipiv[r0:r0 + npiv] = r0 + piv
        ipk = ipiv[r0:r0 + npiv]
        for j in list(range(k)) + list(range(k + 1, nt)):       # swaprows_trail!
            for i in range(k, mt):
                swaprows_trail(T.get(k, j), T.get(i, j), ipk, i, nb)
        akk = T.get(k, k)
        kk = min(akk.shape)
        for j in range(k + 1, nt):                               # TRSM, GEMM
            akj = T.get(k, j)
            akj[:kk, :] = _trsm('L', 'L', 'N', 'U', 1.0, akk[:kk, :kk], akj[:kk, :])
            for i in range(k + 1, mt):
                T.set(i, j, _gemm('N', 'N', -1.0, T.get(i, k), akj[:kk, :], 1.0, T.get(i, j)))
    return F, ipiv, info


def lu_nopivot(A: np.ndarray, nb: int):
    """lu!(A, NoPivot()) (lu.jl:5-54).  Returns (factors, ipiv = 1..min(m, n),
    info of the first tile whose generic_lufact! met a zero pivot)."""
    F = np.array(A, dtype=np.float64, order='F', copy=True)
    m, n = F.shape
    T = TileView(F, nb, nb)
    mt, nt = T.mt, T.nt
    info = 0
    for k in range(min(mt, nt)):
        a, tinfo = generic_lufact_nopivot(T.get(k, k))
        T.set(k, k, a)
        if info == 0 and tinfo != 0:
            info = T.rows[k][0] + tinfo
        akk = T.get(k, k)
        kk = min(akk.shape)
        for i in range(k + 1, mt):
            aik = T.get(i, k)
            aik[:, :kk] = _trsm('R', 'U', 'N', 'N', 1.0, akk[:kk, :kk], aik[:, :kk])
        for j in range(k + 1, nt):
            akj = T.get(k, j)
            akj[:kk, :] = _trsm('L', 'L', 'N', 'U', 1.0, akk[:kk, :kk], akj[:kk, :])
            for i in range(k + 1, mt):
                T.set(i, j, _gemm('N', 'N', -1.0, T.get(i, k), akj[:kk, :], 1.0, T.get(i, j)))
    return F, np.arange(1, min(m, n) + 1, dtype=np.int64), info


def lu(A: np.ndarray, nb: int, pivot: str = 'rowmaximum', check: bool = True,
       allowsingular: bool = False):
    """LinearAlgebra.lu(DA, pivot): the tiled factorization, then
    _check_lu_success (SingularException unless allowsingular)."""
    if check and not np.all(np.isfinite(A)):
        raise ValueError("matrix contains Infs or NaNs")
    if pivot == 'rowmaximum':
        F, ipiv, info = lu_rowmaximum(A, nb)
    else:
        F, ipiv, info = lu_nopivot(A, nb)
    if check and info > 0 and not allowsingular:
        raise SingularException(info)
    return F, ipiv, info


def apply_ipiv_rows(ipiv: np.ndarray, B: np.ndarray, nb: int):
    """_apply_ipiv_rows! (linalg.jl:279-308): for every ipiv chunk k and every
    block i >= k, swaprows_trail!(B[k], B[i]); B in place."""
    TB = TileView(B if B.ndim == 2 else B.reshape(-1, 1, order='F'), nb, max(1, B.shape[1] if B.ndim == 2 else 1))
    mt = TB.mt
    for k in range(mt):
        r0, r1 = TB.rows[k]
        ipk = ipiv[r0:r1]
        for i in range(k, mt):
            for j in range(TB.nt):
                swaprows_trail(TB.get(k, j), TB.get(i, j), ipk, i, nb)
    return B


def ldiv_lu(F: np.ndarray, ipiv: np.ndarray, B: np.ndarray, nb: int):
    """ldiv!(F::LU, B) (linalg.jl:264-278): the rows of B permuted by ipiv,
    then Dagger.trsm! with the unit-lower L and with U.  B (N x r, Fortran
    order) is overwritten and returned."""
    B = np.asfortranarray(B, dtype=np.float64)
    apply_ipiv_rows(ipiv, B, nb)
    if B.ndim == 1:                              # ldiv! of a vector: Dagger.trsv!
        trsv_tiled('L', 'N', 'U', 1.0, F, B, nb)
        trsv_tiled('U', 'N', 'N', 1.0, F, B, nb)
    else:
        trsm_tiled('L', 'L', 'N', 'U', 1.0, F, B, nb)
        trsm_tiled('L', 'U', 'N', 'N', 1.0, F, B, nb)
    return B


def panel_row_list(ipiv_k: np.ndarray, row0: int):
    """One panel's interchanges as the (destination, source) row list the CUDA
    path applies to every other block column, rows counted from row0: the
    interchanges replayed on the contents of the first len(ipiv_k) rows and
    of the rows below them that the pivots reach.  Restated here so that the
    tests pin it against the reference's pair-by-pair swaprows_trail!."""
    npiv = len(ipiv_k)
    top = list(range(npiv))
    below = {}
    for p, g in enumerate(ipiv_k):
        r = int(g) - 1 - row0
        if r == p:
            continue
        if r < npiv:
            top[p], top[r] = top[r], top[p]
        else:
            below.setdefault(r, r)
            top[p], below[r] = below[r], top[p]
    out = [(p, top[p]) for p in range(npiv) if top[p] != p]
    out += [(r, v) for r, v in below.items() if v != r]
    return out


def apply_row_list(L, X: np.ndarray):
    """X[dst] = X[src] for every pair, all sources read before any write."""
    if not L:
        return X
    dst = np.array([d for d, _ in L])
    src = np.array([s for _, s in L])
    X[dst, ...] = X[src, ...].copy()
    return X


def permutation(ipiv: np.ndarray, m: int) -> np.ndarray:
    """perm[t] = the row of A at row t of P A."""
    perm = np.arange(m)
    for p, g in enumerate(ipiv):
        r = int(g) - 1
        perm[p], perm[r] = perm[r], perm[p]
    return perm


def factors_LU(F: np.ndarray):
    m, n = F.shape
    k = min(m, n)
    L = np.tril(F[:, :k], -1) + np.eye(m, k)
    U = np.triu(F[:k, :])
    return L, U


def lu_residual(A: np.ndarray, F: np.ndarray, ipiv: np.ndarray) -> float:
    """||P A - L U||_F / ||A||_F."""
    L, U = factors_LU(F)
    PA = A[permutation(ipiv, A.shape[0]), :]
    return float(np.linalg.norm(PA - L @ U) / np.linalg.norm(A))


def rand_uniform(m: int, n: int, seed: int) -> np.ndarray:
    """rand(m, n): i.i.d. uniform [0, 1) (numpy PCG64(seed)), the reference
    benchmark's and tests' LU input."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.asfortranarray(rng.random((m, n)))
