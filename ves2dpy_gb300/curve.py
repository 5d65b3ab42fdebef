"""Curve calculus on the device (reference: mytorch/curve_batch_compile.py)."""
from __future__ import annotations

import ctypes

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

    def ellipse(self, N, ra, device=None):
        """Ellipse of reduced area ``ra`` with N points (curve_batch_compile.py:494-527).

        Same steps as the reference: the first shape is (a cos t, sin t) with
        a = (1 - sqrt(1 - ra^2)) / ra, accepted when its reduced area is within
        1e-4 (relative); otherwise up to 10 rescalings of a (x 0.9 or x 1.05)
        of the shape (cos t, a sin t), accepted within 1e-2 (absolute).  The
        reduced areas come from ``geomProp`` on the device.  Returns [2N, 1].
        """
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        ra = torch.as_tensor(ra, dtype=torch.float64, device=dev).reshape(-1)[:1]
        t = torch.arange(N, dtype=torch.float64, device=dev) * 2 * torch.pi / N
        a = (1 - torch.sqrt(1 - ra ** 2)) / ra
        X0 = torch.cat((a * torch.cos(t), torch.sin(t)))[:, None]
        ra_new = self.geomProp(X0)[0]
        cond = bool((torch.abs(ra_new - ra) / ra < 1e-4).item())
        it = 0
        while not cond and it < 10:
            it += 1
            if bool((ra_new > ra).item()):
                a = a * 0.9
            else:
                a = a * 1.05
            X0 = torch.cat((torch.cos(t), a * torch.sin(t)))[:, None]
            ra_new = self.geomProp(X0)[0]
            cond = bool((torch.abs(ra_new - ra) < 1e-2).item())
        return X0

    # -- post-step conditioning -------------------------------------------------
    def getPhysicalCenter(self, X):
        """Physical centre (2, nv) (curve_batch_compile.py:84-100)."""
        c, _ = self._center_angle(X)
        return c

    def getIncAngle(self, X):
        """Inclination angle in [0, pi] (curve_batch_compile.py:105-194)."""
        _, a = self._center_angle(X)
        return a

    def _center_angle(self, X):
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = nat.context(N, X.device)
        Xv = to_vm(X)
        c = torch.empty(nv, 2, dtype=torch.float64, device=X.device)
        a = torch.empty(nv, dtype=torch.float64, device=X.device)
        nat.check(ctx.lib.ves_center_angle(ctx.handle, nv, Xv.data_ptr(), c.data_ptr(), a.data_ptr(),
                                           nat.stream_ptr(X.device)), "center_angle")
        return c.t().contiguous(), a

    def alignCenterAngle(self, Xorg, X):
        """Rigid motion of X onto the centre and angle of Xorg (curve_batch_compile.py:842-901)."""
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = nat.context(N, X.device)
        Xo, Xv = to_vm(as_device_f64(Xorg)), to_vm(X)
        out = torch.empty_like(Xv)
        nat.check(ctx.lib.ves_align_center_angle(ctx.handle, nv, Xo.data_ptr(), Xv.data_ptr(), out.data_ptr(),
                                                 nat.stream_ptr(X.device)), "alignCenterAngle")
        return from_vm(out)

    def redistributeArcLength(self, X, modes=None):
        """One equi-arclength pass (curve_batch_compile.py:905-972).  Like the
        reference, ``X`` is updated in place when it is a float64 CUDA tensor;
        returns (X, allGood)."""
        Xd = as_device_f64(X)
        N, nv = Xd.shape[0] // 2, Xd.shape[1]
        if modes is not None:
            m = torch.as_tensor(modes).cpu()
            ref = torch.cat((torch.arange(0, N // 2), torch.arange(-N // 2, 0)))
            if m.numel() != N or not torch.equal(m.to(ref.dtype), ref):
                raise ValueError("redistributeArcLength: modes must be [0..N/2-1, -N/2..-1]")
        ctx = nat.context(N, Xd.device)
        Xv = to_vm(Xd)
        out = torch.empty_like(Xv)
        flags = torch.empty(nv, dtype=torch.int32, device=Xd.device)
        good = ctypes.c_int(0)
        ws = ctx.workspace(ctx.lib.ves_redistribute_arclength_workspace(ctx.handle, nv))
        nat.check(ctx.lib.ves_redistribute_arclength(ctx.handle, nv, Xv.data_ptr(), out.data_ptr(),
                                                     flags.data_ptr(), ctypes.byref(good), ws.data_ptr(),
                                                     ws.numel(), nat.stream_ptr(Xd.device)), "redistributeArcLength")
        res = from_vm(out)
        if X is Xd:
            X.copy_(res)
            res = X
        return res, bool(good.value)

    def correctAreaAndLengthAugLag(self, X, area0, length0):
        """Nearest shape with the original area and length, for vesicles off by
        more than 1e-2 (curve_batch_compile.py:590-710)."""
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = nat.context(N, X.device)
        Xv = to_vm(X)
        a0 = as_device_f64(area0, X.device).contiguous()
        l0 = as_device_f64(length0, X.device).contiguous()
        out = torch.empty_like(Xv)
        ws = ctx.workspace(ctx.lib.ves_correct_area_length_workspace(ctx.handle, nv))
        it = ctypes.c_int(0)
        nat.check(ctx.lib.ves_correct_area_length(ctx.handle, nv, Xv.data_ptr(), a0.data_ptr(), l0.data_ptr(),
                                                  out.data_ptr(), ctypes.byref(it), ws.data_ptr(), ws.numel(),
                                                  nat.stream_ptr(X.device)), "correctAreaAndLengthAugLag")
        self.last_auglag_iters = it.value
        return from_vm(out)
