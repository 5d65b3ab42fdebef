"""Curve calculus on the device (reference: mytorch/curve_batch_compile.py)."""
from __future__ import annotations

import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, to_vm


class Curve:
    """Subset of ``Curve`` used by the BIEM step (curve_batch_compile.py:19-1200)."""

    def getXY(self, X):
        """curve_batch_compile.py:37-40."""
        N = X.shape[0] // 2
        return X[:N, :], X[N:, :]

    def setXY(self, x, y):
        """curve_batch_compile.py:43-49."""
        return torch.cat([x, y], dim=0)

    def diffProp(self, X):
        """Jacobian, unit tangent and curvature (curve_batch_compile.py:400-423)."""
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = nat.context(N, X.device)
        Xv = to_vm(X)
        sa = torch.empty(nv, N, dtype=torch.float64, device=X.device)
        tang = torch.empty(nv, 2 * N, dtype=torch.float64, device=X.device)
        cur = torch.empty(nv, N, dtype=torch.float64, device=X.device)
        nat.check(ctx.lib.ves_diff_prop(ctx.handle, 0, nv, Xv.data_ptr(), sa.data_ptr(), tang.data_ptr(),
                                        cur.data_ptr(), nat.stream_ptr(X.device)), "diffProp")
        return from_vm(sa), from_vm(tang), from_vm(cur)

    def geomProp(self, X):
        """Reduced area, area and length (curve_batch_compile.py:455-473)."""
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = nat.context(N, X.device)
        Xv = to_vm(X)
        out = torch.empty(3, nv, dtype=torch.float64, device=X.device)
        nat.check(ctx.lib.ves_geom_prop(ctx.handle, nv, Xv.data_ptr(), out[0].data_ptr(), out[1].data_ptr(),
                                        out[2].data_ptr(), nat.stream_ptr(X.device)), "geomProp")
        return out[0], out[1], out[2]
