"""DArray and Blocks: the tiled container the Cholesky path receives.

Mirrors Dagger.jl's `DArray{T,N}` with `Blocks(nb, nb)` partitioning
(src/array/darray.jl:107-152) for the part the factor-and-solve path uses:
`distribute` / `DArray(A, Blocks)` (darray.jl:606-629), `DArray{T}(undef,
Blocks, dims)` (darray.jl:633-640), `chunks[i, j]`, `collect`, and `copy`
(`cholcopy`, src/array/cholesky.jl:1).

HBM layout: all tiles of one DArray live in a single device allocation.
Tile (i, j) occupies the slot i + j*mt (column-major tile grid) of
nb_r * nb_c elements and is itself column-major with leading dimension equal
to its row count, so every tile is one contiguous block (a Julia Array chunk)
and the last row/column of tiles may be ragged.  Slots are nb_r*nb_c*8 bytes,
which keeps every tile 256-byte aligned when nb is a multiple of 8.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch


class Blocks:
    """Blocks(nb...): block size per dimension (darray.jl:107-117)."""

    def __init__(self, *blocksize: int):
        if len(blocksize) == 1 and isinstance(blocksize[0], (tuple, list)):
            blocksize = tuple(blocksize[0])
        if not blocksize or any(int(b) <= 0 for b in blocksize):
            raise ValueError("Blocks sizes must be positive")
        self.blocksize = tuple(int(b) for b in blocksize)

    def __eq__(self, other):
        return isinstance(other, Blocks) and self.blocksize == other.blocksize

    def __repr__(self):
        return f"Blocks{self.blocksize}"


def block_ranges(n: int, nb: int):
    return [(s, min(s + nb, n)) for s in range(0, n, nb)]


class DArray:
    """A 1-D or 2-D FP64 array split into device tiles by Blocks."""

    def __init__(self, shape: Sequence[int], part: Blocks, device=None,
                 dtype: torch.dtype = torch.float64, storage: torch.Tensor | None = None):
        shape = tuple(int(s) for s in shape)
        if len(shape) not in (1, 2):
            raise ValueError("DArray supports 1-D and 2-D arrays")
        if len(part.blocksize) != len(shape):
            raise ValueError(f"{part} does not match a {len(shape)}-D array")
        self.shape = shape
        self.partitioning = part
        self.dtype = dtype
        self.device = torch.device(device if device is not None else "cuda")
        self.row_ranges = block_ranges(shape[0], part.blocksize[0])
        self.col_ranges = block_ranges(shape[1], part.blocksize[1]) if len(shape) == 2 else [(0, 1)]
        self.mt, self.nt = len(self.row_ranges), len(self.col_ranges)
        nbr = part.blocksize[0]
        nbc = part.blocksize[1] if len(shape) == 2 else 1
        self.slot = nbr * nbc
        nslots = self.mt * self.nt
        if storage is None:
            storage = torch.empty(max(nslots * self.slot, 1), dtype=dtype, device=self.device)
        self.storage = storage
        self._ptrs = None

    # -- geometry -----------------------------------------------------------
    @property
    def ndim(self):
        return len(self.shape)

    def tile_shape(self, i: int, j: int = 0):
        r0, r1 = self.row_ranges[i]
        c0, c1 = self.col_ranges[j]
        return r1 - r0, c1 - c0

    def tile(self, i: int, j: int = 0) -> torch.Tensor:
        """Chunk (i, j) as a column-major view (strides (1, rows))."""
        r, c = self.tile_shape(i, j)
        off = (i + j * self.mt) * self.slot
        if self.ndim == 1:
            return self.storage.narrow(0, off, r)
        return self.storage.as_strided((r, c), (1, max(r, 1)), off)

    @property
    def chunks(self):
        """mt x nt nested list of tile views (DArray.chunks)."""
        return [[self.tile(i, j) for j in range(self.nt)] for i in range(self.mt)]

    def tile_ptrs(self):
        """ctypes array of device pointers, column-major tile grid (tiles[i + j*mt])."""
        if self._ptrs is None:
            base = self.storage.data_ptr()
            es = self.storage.element_size()
            arr = (ctypes.c_void_p * (self.mt * self.nt))()
            for j in range(self.nt):
                for i in range(self.mt):
                    arr[i + j * self.mt] = base + (i + j * self.mt) * self.slot * es
            self._ptrs = arr
        return self._ptrs

    # -- construction ---------------------------------------------------------
    @classmethod
    def undef(cls, part: Blocks, shape, device=None, dtype=torch.float64):
        """DArray{T}(undef, Blocks, dims) (darray.jl:633-640)."""
        return cls(shape, part, device=device, dtype=dtype)

    @classmethod
    def zeros(cls, part: Blocks, shape, device=None, dtype=torch.float64):
        A = cls(shape, part, device=device, dtype=dtype)
        A.storage.zero_()
        return A

    @classmethod
    def from_array(cls, A, part: Blocks, device=None, dtype=torch.float64):
        """DArray(A, Blocks) / distribute (darray.jl:606-629).  A may be a numpy
        array (copied host to device) or a torch tensor on any device."""
        if isinstance(A, np.ndarray):
            t = torch.from_numpy(np.ascontiguousarray(A))
        else:
            t = A
        D = cls(tuple(t.shape), part, device=device if device is not None else
                (t.device if t.is_cuda else None), dtype=dtype)
        D.copy_from(t)
        return D

    def copy_from(self, t: torch.Tensor):
        """Fills the tiles from a dense (row-major torch) array of the same shape."""
        if tuple(t.shape) != self.shape:
            raise ValueError(f"shape {tuple(t.shape)} != {self.shape}")
        t = t.to(device=self.device, dtype=self.dtype, non_blocking=True)
        if self.ndim == 1:
            for i in range(self.mt):
                r0, r1 = self.row_ranges[i]
                self.tile(i).copy_(t[r0:r1])
            return self
        nbr, nbc = self.partitioning.blocksize
        n0, n1 = self.shape
        if n0 % nbr == 0 and n1 % nbc == 0 and self.slot * self.mt * self.nt == self.storage.numel():
            # one strided copy: tile (i, j) column-major = A[i-block, j-block]^T
            src = t.view(self.mt, nbr, self.nt, nbc).permute(2, 0, 3, 1)
            self.storage.view(self.nt, self.mt, nbc, nbr).copy_(src)
        else:
            for j in range(self.nt):
                c0, c1 = self.col_ranges[j]
                for i in range(self.mt):
                    r0, r1 = self.row_ranges[i]
                    self.tile(i, j).copy_(t[r0:r1, c0:c1])
        return self

    def collect(self) -> torch.Tensor:
        """Dense row-major torch tensor on the array's device (collect(DA))."""
        if self.ndim == 1:
            out = torch.empty(self.shape, dtype=self.dtype, device=self.device)
            for i in range(self.mt):
                r0, r1 = self.row_ranges[i]
                out[r0:r1] = self.tile(i)
            return out
        out = torch.empty(self.shape, dtype=self.dtype, device=self.device)
        nbr, nbc = self.partitioning.blocksize
        n0, n1 = self.shape
        if n0 % nbr == 0 and n1 % nbc == 0 and self.slot * self.mt * self.nt == self.storage.numel():
            out.view(self.mt, nbr, self.nt, nbc).copy_(
                self.storage.view(self.nt, self.mt, nbc, nbr).permute(1, 3, 0, 2))
            return out
        for j in range(self.nt):
            c0, c1 = self.col_ranges[j]
            for i in range(self.mt):
                r0, r1 = self.row_ranges[i]
                out[r0:r1, c0:c1] = self.tile(i, j)
        return out

    def numpy(self) -> np.ndarray:
        return self.collect().cpu().numpy()

    def copy(self) -> "DArray":
        """copy(A): a new DArray with the same partitioning (cholcopy)."""
        D = DArray(self.shape, self.partitioning, device=self.device, dtype=self.dtype)
        D.storage.copy_(self.storage)
        return D

    def __repr__(self):
        return f"DArray{self.shape} {self.partitioning} on {self.device}"


def distribute(A, part: Blocks, device=None) -> DArray:
    return DArray.from_array(A, part, device=device)
