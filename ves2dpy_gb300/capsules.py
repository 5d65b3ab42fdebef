"""Per-vesicle operators on the device (reference: mytorch/capsules.py)."""
from __future__ import annotations

import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, mats_from_vm, to_vm


class capsules:  # noqa: N801 - the reference class name
    """capsules(X, sigma, u, kappa, viscCont) (capsules.py:19-52).

    Holds the geometry of ``X[2N, nv]`` (jacobian ``sa``, unit tangent ``xt``,
    curvature ``cur``, ``isa = 1/sa``, minimum ``length``) both in the
    reference layout and in the device layout used by the kernels.
    """

    def __init__(self, X, sigma, u, kappa, viscCont):
        X = as_device_f64(X)
        self.N = X.shape[0] // 2
        self.nv = X.shape[1]
        self.X = X
        self.sig = sigma
        self.u = u
        self.kappa = kappa
        self.viscCont = viscCont
        self._ctx = nat.context(self.N, X.device)
        dev = X.device
        self._Xv = to_vm(X)
        N, nv = self.N, self.nv
        self._sa = torch.empty(nv, N, dtype=torch.float64, device=dev)
        self._tang = torch.empty(nv, 2 * N, dtype=torch.float64, device=dev)
        self._cur = torch.empty(nv, N, dtype=torch.float64, device=dev)
        lib, h, st = self._ctx.lib, self._ctx.handle, nat.stream_ptr(dev)
        nat.check(lib.ves_diff_prop(h, 0, nv, self._Xv.data_ptr(), self._sa.data_ptr(), self._tang.data_ptr(),
                                    self._cur.data_ptr(), st), "capsules")
        self._isa = 1.0 / self._sa
        self.sa = from_vm(self._sa)
        self.xt = from_vm(self._tang)
        self.cur = from_vm(self._cur)
        self.isa = 1.0 / self.sa
        geo = torch.empty(3, nv, dtype=torch.float64, device=dev)
        nat.check(lib.ves_geom_prop(h, nv, self._Xv.data_ptr(), geo[0].data_ptr(), geo[1].data_ptr(),
                                    geo[2].data_ptr(), st), "capsules length")
        self.length = torch.min(geo[2])

    # -- traction and divergence ------------------------------------------------
    def _trac(self, Xv, sigv, kappa):
        N, nv = self.N, self.nv
        f = torch.empty(nv, 2 * N, dtype=torch.float64, device=self.X.device)
        nat.check(self._ctx.lib.ves_trac_jump(self._ctx.handle, nv, float(kappa), self._isa.data_ptr(),
                                              self._tang.data_ptr(), Xv.data_ptr(), 2 * N, sigv.data_ptr(), N,
                                              f.data_ptr(), nat.stream_ptr(self.X.device)), "tracJump")
        return f

    def tracJump(self, f, sigma):
        """-kappa d^4 f/ds^4 + d/ds(sigma x_s)  (capsules.py:54-60)."""
        fv = to_vm(as_device_f64(f))
        sv = to_vm(as_device_f64(sigma))
        return from_vm(self._trac(fv, sv, self.kappa))

    def bendingTerm(self, f):
        """capsules.py:62-68."""
        fv = to_vm(as_device_f64(f))
        return from_vm(self._trac(fv, torch.zeros(self.nv, self.N, dtype=torch.float64, device=fv.device),
                                  self.kappa))

    def tensionTerm(self, sig):
        """capsules.py:70-80."""
        sv = to_vm(as_device_f64(sig))
        return from_vm(self._trac(torch.zeros(self.nv, 2 * self.N, dtype=torch.float64, device=sv.device), sv, 0.0))

    def surfaceDiv(self, f):
        """capsules.py:82-89."""
        fv = to_vm(as_device_f64(f))
        N, nv = self.N, self.nv
        out = torch.empty(nv, N, dtype=torch.float64, device=fv.device)
        nat.check(self._ctx.lib.ves_surface_div(self._ctx.handle, nv, self._isa.data_ptr(), self._tang.data_ptr(),
                                                fv.data_ptr(), 2 * N, out.data_ptr(), N,
                                                nat.stream_ptr(fv.device)), "surfaceDiv")
        return from_vm(out)

    def computeDerivs(self):
        """Ben (2N,2N,nv), Ten (2N,N,nv), Div (N,2N,nv) (capsules.py:91-206)."""
        N, nv, dev = self.N, self.nv, self.X.device
        Ben = torch.empty(nv, 2 * N, 2 * N, dtype=torch.float64, device=dev)
        Ten = torch.empty(nv, 2 * N, N, dtype=torch.float64, device=dev)
        Div = torch.empty(nv, N, 2 * N, dtype=torch.float64, device=dev)
        lib, h = self._ctx.lib, self._ctx.handle
        nbytes = lib.ves_compute_derivs_workspace(h, nv)
        ws = self._ctx.workspace(nbytes)
        nat.check(lib.ves_compute_derivs(h, nv, self._isa.data_ptr(), self._tang.data_ptr(), Ben.data_ptr(),
                                         Ten.data_ptr(), Div.data_ptr(), ws.data_ptr(), ws.numel(),
                                         nat.stream_ptr(dev)), "computeDerivs")
        return mats_from_vm(Ben), mats_from_vm(Ten), mats_from_vm(Div)

    def repulsionForce(self, X, W, eta):
        """Penalty-layer repulsion between vesicles (capsules.py:209-252):
        for each point, W * sum over the points of the other vesicles of
        dF(d) (x - y) with L = floor(eta / d) layers, d = sqrt(|x - y|^2 + 1e-10).
        Returns [2N, nv]."""
        X = as_device_f64(X)
        N, nv = X.shape[0] // 2, X.shape[1]
        Xv = to_vm(X)
        out = torch.empty_like(Xv)
        lib = nat.load_library()
        ws = torch.empty(lib.ves_repulsion_force_workspace(nv), dtype=torch.uint8, device=X.device)
        nat.check(lib.ves_repulsion_force(N, nv, Xv.data_ptr(), float(W), float(eta), out.data_ptr(), ws.data_ptr(),
                                          ws.numel(), nat.stream_ptr(X.device)), "repulsionForce")
        return from_vm(out)

    def getZone(self, vesicle2=None, relate=1):
        """Near zone of every vesicle w.r.t. every other, MATLAB getZone semantics
        (matlab/capsules_py.m:194-467, relate == 1; absent from the Python
        reference, which calls it at tstep_biem.py:209-217)."""
        if relate != 1 or vesicle2 is not None:
            raise NotImplementedError("getZone: only vesicle-to-vesicle zones (relate=1)")
        from .biem_support import NearZone
        return NearZone.build_matlab(self._Xv, self.N)
