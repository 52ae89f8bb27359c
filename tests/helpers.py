"""Shared helpers for the tests (column-major device tensors, tolerances)."""
import numpy as np

FP64_RTOL = 1e-13  # plain FP64 path vs the oracle, normwise relative


def dev_f(a):
    """Fortran-ordered numpy matrix -> column-major float64 CUDA tensor."""
    import torch
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return torch.from_numpy(a.copy()).cuda()
    r, c = a.shape
    t = torch.empty((c, r), dtype=torch.float64, device="cuda")
    t.copy_(torch.from_numpy(np.ascontiguousarray(a.T)))
    return t.T


def host_f(t):
    """Column-major CUDA tensor -> Fortran-ordered numpy array."""
    if t.dim() == 1:
        return t.cpu().numpy()
    return np.asfortranarray(t.T.cpu().numpy().T)


def rel_err(x, ref):
    x = np.asarray(x)
    ref = np.asarray(ref)
    s = np.abs(ref).max()
    return float(np.abs(x - ref).max() / (s if s > 0 else 1.0))
