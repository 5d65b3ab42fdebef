"""Layer potentials on the device (reference: mytorch/poten.py)."""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat
from .biem_support import NearZone, _farfield, _density, upsample_factor
from .capsules import capsules
from .layout import as_device_f64, from_vm, mats_from_vm, mats_to_vm, to_vm

LAGRANGE_INTERP = [
    [64.80, -388.80, 972.00, -1296.00, 972.00, -388.80, 64.80],
    [-226.80, 1296.00, -3078.00, 3888.00, -2754.00, 1036.80, -162.00],
    [315.00, -1674.00, 3699.00, -4356.00, 2889.00, -1026.00, 153.00],
    [-220.50, 1044.00, -2074.50, 2232.00, -1381.50, 468.00, -67.50],
    [81.20, -313.20, 526.50, -508.00, 297.00, -97.20, 13.70],
    [-14.70, 36.00, -45.00, 40.00, -22.50, 7.20, -1.00],
    [1.00, 0.00, 0.00, 0.00, 0.00, 0.00, 0.00]]


def visc_tensor(viscCont, nv, device):
    """Viscosity contrasts as a device float64 vector of nv entries."""
    v = torch.as_tensor(1.0 if viscCont is None else viscCont, dtype=torch.float64)
    if v.dim() == 0:
        v = v.repeat(nv)
    v = v.reshape(-1)
    if v.numel() != nv:
        raise ValueError(f"viscCont has {v.numel()} entries for {nv} vesicles")
    return v.to(device).contiguous()


def _is_double_layer(kernel) -> bool:
    f = getattr(kernel, "__func__", kernel)
    return f is Poten.exactStokesDL or getattr(f, "__name__", "") == "exactStokesDL"


class Poten:
    """Poten(N) (poten.py:14-37): the quadrature tables live in the device
    context of the C library, created once per (N, device)."""

    def __init__(self, N, device=None):
        self.N = int(N)
        self.Nup = upsample_factor(self.N)
        self.device = torch.device(device) if device is not None else torch.device("cuda",
                                                                                    torch.cuda.current_device())
        self._ctx = nat.context(self.N, self.device)
        self.interpMat = torch.tensor(LAGRANGE_INTERP, dtype=torch.float64, device=self.device)

    # -- self interaction --------------------------------------------------------
    def stokesSLmatrix(self, vesicle, precision: str = "fp64"):
        """Alpert single-layer matrix G (2N, 2N, nv) (poten.py:40-99)."""
        ctx, nv = self._ctx, vesicle.nv
        Xv = to_vm(as_device_f64(vesicle.X))
        G = torch.empty(nv, 2 * self.N, 2 * self.N, dtype=torch.float64, device=Xv.device)
        prec = nat.PREC[precision]
        ws = ctx.workspace(ctx.lib.ves_stokes_sl_matrix_workspace(ctx.handle, nv, prec))
        nat.check(ctx.lib.ves_stokes_sl_matrix(ctx.handle, nv, Xv.data_ptr(), prec, G.data_ptr(), ws.data_ptr(),
                                               ws.numel(), nat.stream_ptr(Xv.device)), "stokesSLmatrix")
        return mats_from_vm(G)

    def exactStokesSLdiag(self, vesicle, G, f):
        """Per-vesicle G[:, :, k] @ f[:, k] (poten.py:213-224)."""
        Gv = mats_to_vm(as_device_f64(G))
        fv = to_vm(as_device_f64(f))
        nv, m = Gv.shape[0], Gv.shape[1]
        out = torch.empty(nv, m, dtype=torch.float64, device=fv.device)
        nat.check(nat.load_library().ves_sl_diag(nv, m, Gv.data_ptr(), fv.data_ptr(), out.data_ptr(),
                                                 nat.stream_ptr(fv.device)), "exactStokesSLdiag")
        return from_vm(out)

    def stokesDLmatrix(self, vesicle, precision: str = "fp64"):
        """Double-layer matrix D (2N, 2N, nv) (poten.py:102-175): trapezoid rule
        on the Nup-upsampled curve with the curvature limit on the diagonal,
        restricted to N points; zero for vesicles without a viscosity
        contrast.  ``precision`` "fp32c" does the restriction products in FP32."""
        ctx, nv = self._ctx, vesicle.nv
        Xv = to_vm(as_device_f64(vesicle.X))
        visc = visc_tensor(vesicle.viscCont, nv, Xv.device)
        D = torch.empty(nv, 2 * self.N, 2 * self.N, dtype=torch.float64, device=Xv.device)
        prec = nat.PREC[precision]
        ws = ctx.workspace(ctx.lib.ves_stokes_dl_matrix_workspace(ctx.handle, nv, prec))
        nat.check(ctx.lib.ves_stokes_dl_matrix(ctx.handle, nv, Xv.data_ptr(), visc.data_ptr(), prec, D.data_ptr(),
                                               ws.data_ptr(), ws.numel(), nat.stream_ptr(Xv.device)),
                  "stokesDLmatrix")
        return mats_from_vm(D)

    def exactStokesDLdiag(self, vesicle, D, f):
        """Per-vesicle D[:, :, k] @ f[:, k] (poten.py:227-238)."""
        return self.exactStokesSLdiag(vesicle, D, f)

    # -- between vesicles ------------------------------------------------------
    def exactStokesDL(self, vesicle, f, Xtar=None, K1=None, precision: str = "fp64"):
        """Double layer of vesicles K1 (density f, scaled by 1 - viscCont) at
        every column of Xtar (poten.py:399-441).  ``precision`` "fp64": direct
        FP64 sum; "fp32m": multipole series for the separated vesicle-target
        pairs (at most 128 points per target column), direct FP64 for the rest."""
        Xtar = as_device_f64(Xtar)
        if Xtar.dim() == 1:
            Xtar = Xtar.unsqueeze(1)
        K1 = list(range(vesicle.nv)) if K1 is None else [int(k) for k in K1]
        N, ntp, ncol = vesicle.N, Xtar.shape[0] // 2, Xtar.shape[1]
        dev = Xtar.device
        idx = torch.tensor(K1, dtype=torch.long, device=dev)
        Xs = to_vm(as_device_f64(vesicle.X).index_select(1, idx))
        ts = to_vm(as_device_f64(vesicle.xt).index_select(1, idx))
        fs = to_vm(as_device_f64(f).index_select(1, idx))
        sas = to_vm(as_device_f64(vesicle.sa).index_select(1, idx))
        visc = visc_tensor(vesicle.viscCont, vesicle.nv, dev).index_select(0, idx).contiguous()
        lib, st = nat.load_library(), nat.stream_ptr(dev)
        den = torch.empty_like(fs)
        nat.check(lib.ves_dl_density(len(K1), N, fs.data_ptr(), sas.data_ptr(), visc.data_ptr(), den.data_ptr(), st),
                  "exactStokesDL density")
        Xt = to_vm(Xtar)
        out = torch.empty(ncol, 2 * ntp, dtype=torch.float64, device=dev)
        prec = nat.PREC[precision]
        ws = self._ctx.workspace(lib.ves_farfield_dl_workspace(prec, len(K1), ncol, ntp))
        nat.check(lib.ves_farfield_dl(self._ctx.handle, prec, len(K1), N, Xs.data_ptr(), ts.data_ptr(), den.data_ptr(),
                                      sas.data_ptr(), visc.data_ptr(), ncol, ntp, Xt.data_ptr(), None, None,
                                      out.data_ptr(), ws.data_ptr(), ws.numel(), st), "exactStokesDL")
        return from_vm(out)

    def _near_dl(self, scheme, vesicleSou, f, selfMat, Near, precision="fp64"):
        """nearSingInt with kernelDirect = exactStokesDL on the device."""
        X = as_device_f64(vesicleSou.X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = self._ctx
        Xv = to_vm(X)
        st = nat.stream_ptr(X.device)
        Xup = torch.empty(nv, 2 * self.Nup, dtype=torch.float64, device=X.device)
        sa_up = torch.empty(nv, self.Nup, dtype=torch.float64, device=X.device)
        tang_up = torch.empty(nv, 2 * self.Nup, dtype=torch.float64, device=X.device)
        nat.check(ctx.lib.ves_upsample_geometry(ctx.handle, nv, Xv.data_ptr(), Xup.data_ptr(), sa_up.data_ptr(),
                                                tang_up.data_ptr(), None, st), "upsample geometry")
        visc = visc_tensor(vesicleSou.viscCont, nv, X.device)
        fv = to_vm(as_device_f64(f))
        vself = to_vm(as_device_f64(selfMat(f))) if selfMat is not None else None
        LP = torch.empty(nv, 2 * N, dtype=torch.float64, device=X.device)
        ws = ctx.workspace(ctx.lib.ves_near_sing_int_dl_workspace(ctx.handle, nv))
        stc = Near.struct() if Near is not None else None
        h = Near.h if Near is not None else 0.0
        nat.check(ctx.lib.ves_near_sing_int_dl(ctx.handle, nat.NEAR[scheme], nat.PREC[precision], nv, Xv.data_ptr(),
                                               Xup.data_ptr(),
                                               tang_up.data_ptr(), sa_up.data_ptr(), visc.data_ptr(), fv.data_ptr(),
                                               nat.ptr(vself), ctypes.byref(stc) if stc is not None else None,
                                               float(h), LP.data_ptr(), None, ws.data_ptr(), ws.numel(), st),
                  "nearSingInt (double layer)")
        return from_vm(LP)

    def exactStokesSL(self, vesicle, f, Xtar=None, K1=None, precision: str = "fp64"):
        """Single layer of vesicles K1 at the single target column Xtar (poten.py:280-336)."""
        Xtar = as_device_f64(Xtar)
        if Xtar.dim() == 1:
            Xtar = Xtar.unsqueeze(1)
        if Xtar.shape[1] != 1:
            raise TypeError("ncol != 1")
        K1 = list(range(vesicle.nv)) if K1 is None else list(K1)
        N = vesicle.N
        den = _density(vesicle.sa[:, K1], as_device_f64(f)[:, K1], N, Xtar.device)
        out = _farfield(precision, to_vm(vesicle.X[:, K1]), den, to_vm(Xtar), None, None, Xtar.shape[0] // 2)
        return from_vm(out)

    def _near_common(self, scheme, vesicleSou, f, selfMat, NearV2V, precision):
        X = as_device_f64(vesicleSou.X)
        N, nv = X.shape[0] // 2, X.shape[1]
        ctx = self._ctx
        Xv = to_vm(X)
        Xup = torch.empty(nv, 2 * self.Nup, dtype=torch.float64, device=X.device)
        st = nat.stream_ptr(X.device)
        nat.check(ctx.lib.ves_upsample(ctx.handle, nv, 2, Xv.data_ptr(), Xup.data_ptr(), st), "upsample")
        sa_up = torch.empty(nv, self.Nup, dtype=torch.float64, device=X.device)
        nat.check(ctx.lib.ves_diff_prop(ctx.handle, 1, nv, Xup.data_ptr(), sa_up.data_ptr(), None, None, st),
                  "diffProp up")
        fv = to_vm(as_device_f64(f))
        vself = to_vm(as_device_f64(selfMat(f))) if selfMat is not None else None
        LP = torch.empty(nv, 2 * N, dtype=torch.float64, device=X.device)
        near = torch.empty_like(LP)
        prec = nat.PREC[precision]
        ws = ctx.workspace(ctx.lib.ves_near_sing_int_workspace(ctx.handle, prec, nv))
        stc = NearV2V.struct() if NearV2V is not None else None
        h = NearV2V.h if NearV2V is not None else 0.0
        nat.check(ctx.lib.ves_near_sing_int(ctx.handle, nat.NEAR[scheme], prec, nv, Xv.data_ptr(), sa_up.data_ptr(),
                                            Xup.data_ptr(), fv.data_ptr(), nat.ptr(vself),
                                            ctypes.byref(stc) if stc is not None else None, float(h),
                                            LP.data_ptr(), near.data_ptr(), ws.data_ptr(), ws.numel(), st),
                  "nearSingInt")
        return from_vm(LP), from_vm(near)

    def nearSingInt_hh(self, vesicleSou, f, selfMat, NearV2V, kernelDirect=None, vesicleTar=None, tEqualS=True,
                       precision: str = "fp64"):
        """poten.py:466-600: far field over upsampled sources with the near pairs
        of ``NearV2V`` removed, plus the hedgehog correction.  Returns
        (LP, nearField).  ``kernelDirect`` is replaced by the fused device kernel."""
        if not tEqualS or (vesicleTar is not None and vesicleTar is not vesicleSou):
            raise NotImplementedError("nearSingInt_hh: only sources == targets (tEqualS)")
        if vesicleSou.nv == 1:
            z = torch.zeros_like(as_device_f64(vesicleSou.X))
            return z, z
        if not isinstance(NearV2V, NearZone) or NearV2V.scheme != "py_hh":
            raise TypeError("NearV2V must come from naiveNearZoneInfo")
        if _is_double_layer(kernelDirect):
            return self._near_dl("py_hh", vesicleSou, f, selfMat, NearV2V, precision), None
        return self._near_common("py_hh", vesicleSou, f, selfMat, NearV2V, precision)

    def nearSingInt_rbf(self, vesicleSou, f, selfMat, NearV2V, kernelDirect=None, vesicleTar=None, tEqualS=True,
                        precision: str = "fp64"):
        """poten.py:643-894: far field over upsampled sources with the near pairs
        of ``NearV2V`` removed, plus, for each near pair, the source vesicle's
        Gaussian RBF fit of its self velocity on three layers (the boundary
        with ``selfMat(f)`` and two normal offsets with its own single layer)
        evaluated at the target point.  Returns LP.  ``kernelDirect`` is
        replaced by the device all-pairs kernel."""
        if not tEqualS or (vesicleTar is not None and vesicleTar is not vesicleSou):
            raise NotImplementedError("nearSingInt_rbf: only sources == targets (tEqualS)")
        if vesicleSou.nv == 1:
            return torch.zeros_like(as_device_f64(vesicleSou.X))
        if not isinstance(NearV2V, NearZone) or NearV2V.scheme != "py_hh":
            raise TypeError("NearV2V must come from naiveNearZoneInfo")
        return self._near_common("py_rbf", vesicleSou, f, selfMat, NearV2V, precision)[0]

    def nearSingInt(self, vesicleSou, f, selfMat, NearStruct, kernelDirect=None, vesicleTar=None, tEqualS=True,
                    precision: str = "fp64"):
        """MATLAB nearSingInt (matlab/poten_py.m:495-692) with NearStruct from
        capsules.getZone: trapezoid contribution of the near source removed and
        replaced by the 7-point Lagrange extrapolation along the normal.

        With ``kernelDirect = exactStokesDL`` (the viscosity-contrast calls at
        tstep_biem.py:236,501) the layer potential is the double layer; the
        near lists may then also come from naiveNearZoneInfo (the step's
        ``NearV2V``), whose near pairs get the nearSingInt_hh correction."""
        if not tEqualS or (vesicleTar is not None and vesicleTar is not vesicleSou):
            raise NotImplementedError("nearSingInt: only sources == targets (tEqualS)")
        if vesicleSou.nv == 1:
            return torch.zeros_like(as_device_f64(vesicleSou.X))
        if _is_double_layer(kernelDirect):
            if NearStruct is None:
                return self._near_dl("none", vesicleSou, f, None, None, precision)
            if not isinstance(NearStruct, NearZone):
                raise TypeError("NearStruct must come from capsules.getZone or naiveNearZoneInfo")
            return self._near_dl("matlab" if NearStruct.scheme == "matlab" else "py_hh", vesicleSou, f, selfMat,
                                 NearStruct, precision)
        if NearStruct is None:
            return self._near_common("none", vesicleSou, f, None, None, precision)[0]
        if not isinstance(NearStruct, NearZone) or NearStruct.scheme != "matlab":
            raise TypeError("NearStruct must come from capsules.getZone")
        return self._near_common("matlab", vesicleSou, f, selfMat, NearStruct, precision)[0]
