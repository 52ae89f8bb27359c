"""Mixed-precision Cholesky solve with iterative refinement.

A faster form beside the FP64 drop-in (cholesky / ldiv_), reached from the
same DArray: the factor of the diagonally scaled matrix is computed with
16-bit tensor-core trailing updates (tcgen05, FP32 accumulation), FP32
diagonal blocks with an FP64 retry on a failed pivot and FP32 panel solves;
solutions are refined in FP64 (iterative refinement, switching to GMRES-IR
when refinement stalls) until the normwise backward error of every column is
at most `tol`.  Precisions: 'bf16', 'bf16x3' (hi/lo split, three products),
'bf16x6' (hi/mid/lo split, six products: FP32-accurate tensor-core updates),
'fp8' (E4M3 with a power-of-two scale per vector, one product at twice the
BF16 rate: for well-conditioned matrices), 'fp16', 'fp16x3' (with per-panel
power-of-two scaling) and 'fp32' (CUDA-core FP32 updates).
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import (DG_PREC, DgIrOpts, DgIrReport, DgMixedStats, PosDefException, check, lib)
from .darray import DArray
from .linalg import _stream


def colmajor(B: torch.Tensor) -> torch.Tensor:
    """A column-major (strides (1, n)) FP64 copy/view of an n x r tensor."""
    if B.dim() == 1:
        B = B.unsqueeze(1)
    if B.stride(0) == 1 and B.stride(1) >= B.shape[0]:
        return B
    return B.t().contiguous().t()


class MixedCholesky:
    """Handle of a mixed-precision factor; keeps a reference to the FP64
    DArray (its tiles give the FP64 residuals)."""

    # first diagonal shift tried when the low-precision factorization breaks
    # down (about the operand precision's unit roundoff), grown 10x per retry
    SHIFT0 = {"bf16": 4e-3, "bf16x3": 1e-5, "bf16x6": 1e-7, "fp8": 3e-2, "fp16": 5e-4,
              "fp16x3": 1e-6, "fp32": 1e-7}

    def __init__(self, A: DArray, precision: str = "bf16x3", stream=None, check_: bool = True,
                 auto_shift: bool = True, shift: float = 0.0, max_shift_retries: int = 4):
        """auto_shift: when the factorization of the scaled matrix breaks down
        (a pivot of a matrix too ill-conditioned for the operand precision),
        refactor S A S + shift I with a growing shift; refinement (GMRES-IR)
        then still solves A x = b.  A matrix with a non-positive diagonal
        entry is not positive definite and is reported at once."""
        if A.ndim != 2 or A.shape[0] != A.shape[1]:
            raise ValueError("matrix is not square")
        nb = A.partitioning.blocksize[0]
        if A.partitioning.blocksize[1] != nb:
            raise ValueError("use Blocks(nb, nb)")
        if precision not in DG_PREC:
            raise ValueError(f"precision must be one of {sorted(DG_PREC)}")
        self.A = A
        self.precision = precision
        self.stream = stream
        self.handle = None
        tries = max_shift_retries if auto_shift else 0
        sigma = shift
        while True:
            h = ctypes.c_void_p()
            rc = lib().dg_mixed_factor_ex(ctypes.byref(h), A.shape[0], nb, A.tile_ptrs(),
                                          DG_PREC[precision], float(sigma), _stream(stream))
            self.handle = h.value
            if rc < 0:
                self.close()
                check(rc)
            if rc == 0 or tries == 0 or self._bad_diagonal():
                break
            self.close()
            sigma = self.SHIFT0[precision] if sigma == 0.0 else 10.0 * sigma
            tries -= 1
        self.info = rc
        if rc > 0 and check_:
            self.close()
            raise PosDefException(rc)

    def _bad_diagonal(self) -> bool:
        """True when A itself has a non-positive diagonal entry (not SPD)."""
        d = torch.cat([self.A.tile(i, i).diagonal() for i in range(self.A.mt)])
        return bool((d <= 0).any().item())

    def stats(self) -> dict:
        st = DgMixedStats()
        check(lib().dg_mixed_info(self.handle, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def solve(self, B: torch.Tensor, tol: float = 1e-12, max_iter: int = 30, gmres: str = "auto",
              restart: int = 30, gmres_inner_tol: float = 1e-4, out: torch.Tensor | None = None,
              raise_on_failure: bool = True, stream=None):
        """X = A^-1 B in FP64 (B: n or n x r CUDA tensor).  Returns (X, report).
        Runs on `stream` (default: the stream the factor was made on)."""
        n = self.A.shape[0]
        vec = B.dim() == 1
        Bc = colmajor(B.to(torch.float64))
        r = Bc.shape[1]
        X = out if out is not None else torch.empty((r, n), dtype=torch.float64,
                                                    device=Bc.device).t()
        o = DgIrOpts(tol, max_iter, {"auto": 0, "always": 1, "never": 2}[gmres], restart,
                     gmres_inner_tol)
        rep = DgIrReport()
        # a single column's stride is arbitrary in torch; any ld >= n is valid
        ldb = Bc.stride(1) if r > 1 else max(Bc.stride(1), n)
        ldx = X.stride(1) if r > 1 else max(X.stride(1), n)
        rc = lib().dg_mixed_solve(self.handle, r, Bc.data_ptr(), ldb, X.data_ptr(),
                                  ldx, ctypes.byref(o), ctypes.byref(rep),
                                  _stream(stream if stream is not None else self.stream))
        report = {f: getattr(rep, f) for f, _ in rep._fields_}
        if rc != 0 and (raise_on_failure or rc != -1004):
            check(rc)
        return (X[:, 0] if vec else X), report

    def close(self):
        if getattr(self, "handle", None):
            lib().dg_mixed_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cholesky_mixed(A: DArray, precision: str = "bf16x3", stream=None, check_: bool = True,
                   **kwargs):
    """The mixed-precision factor of a DArray (see MixedCholesky)."""
    return MixedCholesky(A, precision, stream, check_, **kwargs)
