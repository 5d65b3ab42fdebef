"""Fourier resampling on the device (reference: mytorch/filter.py)."""
from __future__ import annotations

import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, to_vm


def interpft_vec(X, N_new: int):
    """Resample x and y rows from N to N_new = N*ceil(sqrt(N)) points
    (filter.py:192-194 with the interpft convention of :221-249)."""
    X = as_device_f64(X)
    N, nv = X.shape[0] // 2, X.shape[1]
    if N_new == N:
        return X.clone()
    ctx = nat.context(N, X.device)
    if N_new != ctx.Nup:
        raise NotImplementedError("interpft_vec: the device path resamples N -> N*ceil(sqrt(N)) only")
    Xv = to_vm(X)
    out = torch.empty(nv, 2 * N_new, dtype=torch.float64, device=X.device)
    nat.check(ctx.lib.ves_upsample(ctx.handle, nv, 2, Xv.data_ptr(), out.data_ptr(), nat.stream_ptr(X.device)),
              "interpft_vec")
    return from_vm(out)


def upsample_fft(x, N_new: int):
    """filter.py:7-27 (same operator as interpft_vec for upsampling)."""
    return interpft_vec(x, N_new)
