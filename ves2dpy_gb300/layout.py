"""Conversions between the reference layout and the device layout.

The reference stores curves as ``X[2N, nv]`` (x rows, then y rows, one column
per vesicle).  The kernels read vesicle-major ``[nv][2][N]`` float64 arrays,
which is exactly ``X.T`` made contiguous.
"""
from __future__ import annotations

import torch


def as_device_f64(t: torch.Tensor, device=None) -> torch.Tensor:
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if device is not None:
        t = t.to(device)
    if t.device.type != "cuda":
        raise ValueError("ves2dpy_gb300 operators take CUDA tensors (got %s)" % t.device)
    return t.to(torch.float64)


def to_vm(X: torch.Tensor) -> torch.Tensor:
    """[rows, nv] (reference) -> [nv, rows] contiguous (device layout)."""
    if X.dim() == 1:
        X = X.unsqueeze(1)
    return X.to(torch.float64).t().contiguous()


def from_vm(V: torch.Tensor) -> torch.Tensor:
    """[nv, rows] -> [rows, nv] (reference layout, contiguous)."""
    return V.t().contiguous()


def mats_to_vm(M: torch.Tensor) -> torch.Tensor:
    """(r, c, nv) reference stack of matrices -> [nv][r][c] contiguous."""
    return M.to(torch.float64).permute(2, 0, 1).contiguous()


def mats_from_vm(M: torch.Tensor) -> torch.Tensor:
    """[nv][r][c] -> (r, c, nv)."""
    return M.permute(1, 2, 0).contiguous()
