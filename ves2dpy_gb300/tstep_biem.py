"""Implicit BIEM time stepper on one GPU (reference: mytorch/tstep_biem.py).

``TStepBiem(X, Xwalls, options, prams)`` and ``time_step(X, sigma, eta, RS)``
keep the reference signatures and return values; the whole step (geometry,
Alpert matrix, near lists, block preconditioner, GMRES with its matvecs) runs
in one call to ``ves_biem_step`` of the C library.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, to_vm


class TStepBiem:
    """tstep_biem.py:25-153.

    With a viscosity contrast (``prams['viscCont'] != 1``) the step adds the
    double-layer terms of the reference (D, Fdlp, alpha = (1 + visc)/2); the
    double layer's near pairs use the py_hh rule with the naiveNearZoneInfo
    lists ("py_hh", "py_rbf") or the MATLAB rule ("matlab").

    Extra keyword options select the device arithmetic:
    ``near`` ("py_hh" = the reference's nearSingInt_hh, "py_rbf" = its
    nearSingInt_rbf as in the newtorch step, "matlab" = the MATLAB
    near-singular scheme, "none"), ``farfield_precision`` and ``sl_precision``
    ("fp64" or "fp32c").
    """

    def __init__(self, X, Xwalls, options, prams, near: str = "py_hh", farfield_precision: str = "fp32c",
                 sl_precision: str = "fp32c", device=None, precond_precision: str = "fp64"):
        if Xwalls is not None:
            raise NotImplementedError("confined flows (walls) are not supported by the device stepper")
        X = as_device_f64(X, device)
        self.device = X.device
        self.N = X.shape[0] // 2
        self.nv = X.shape[1]
        self.Xwalls = None
        self.dt = float(prams["dt"])
        self.kappa = float(prams["kappa"])
        self.viscCont = prams.get("viscCont")
        # viscosity contrast (tstep_biem.py:195-244): double-layer terms when any vesicle has visc != 1
        from .poten import visc_tensor
        visc = visc_tensor(self.viscCont, self.nv, self.device)
        self._visc = visc if bool(torch.any(visc != 1)) else None
        self.gmresTol = float(prams["gmresTol"])
        self.gmresMaxIter = int(prams["gmresMaxIter"])
        self.farFieldSpeed = float(prams.get("farFieldSpeed", 1.0))
        self.chanWidth = float(prams.get("chanWidth", 1.0))
        self.vortexSize = float(prams.get("vortexSize", 1.0))
        self.options = dict(options)
        self.usePreco = bool(options.get("usePreco", True))
        self.confined = False
        # repulsion (tstep_biem.py:75-83), off for a single vesicle
        self.repulsion = bool(options.get("repulsion", False)) and X.shape[1] > 1
        self.repStrength = float(prams.get("repStrength", 900))
        self.minDist = float(prams.get("minDist", 0.4))
        if self.repulsion and near not in ("py_hh", "py_rbf"):
            raise NotImplementedError("repulsion needs near='py_hh' or 'py_rbf' (naiveNearZoneInfo lists)")
        self.near = near
        if precond_precision not in ("fp64", "fp32"):
            raise ValueError("precond_precision: 'fp64' or 'fp32'")
        self.precond_precision = precond_precision
        self.farfield_precision = farfield_precision
        self.sl_precision = sl_precision
        from .poten import Poten
        from .curve import Curve
        self.op = Poten(self.N, self.device)
        _, self.area, self.length = Curve().geomProp(X)
        self._ctx = nat.context(self.N, self.device)
        self.last = None
        # near-list capacities (candidates per vesicle, MATLAB entries; 0 =
        # the library default); they grow when a step reports more
        self._maxc = 32
        self._maxe = 0

    def params(self) -> nat.StepParams:
        p = nat.StepParams()
        p.dt = self.dt
        p.kappa = self.kappa
        p.gmres_tol = self.gmresTol
        p.gmres_maxiter = self.gmresMaxIter
        p.gmres_restart = 20
        p.use_preco = (2 if self.precond_precision == "fp32" else 1) if self.usePreco else 0
        flow = self.options.get("farField", "shear")
        if flow not in nat.FLOW:
            raise ValueError("Unknown or missing flow type in bg_flow.")
        p.flow = nat.FLOW[flow]
        p.speed = self.farFieldSpeed
        p.chan_width = self.chanWidth
        p.vortex_size = self.vortexSize
        p.near_scheme = nat.NEAR[self.near]
        p.farfield_precision = nat.PREC[self.farfield_precision]
        p.sl_precision = nat.PREC[self.sl_precision]
        p.maxc = self._maxc
        p.max_entries = self._maxe
        p.repulsion = 1 if self.repulsion else 0
        p.rep_strength = self.repStrength
        p.min_dist = self.minDist
        p.visc_cont = None if self._visc is None else self._visc.data_ptr()
        return p

    def workspace_bytes(self) -> int:
        p = self.params()
        return int(self._ctx.lib.ves_biem_step_workspace(self._ctx.handle, ctypes.byref(p), self.nv))

    def step_device(self, Xv, sigv, Xout=None, sigout=None, ws=None):
        """One step on device-layout tensors Xv[nv][2N], sigv[nv][N] (float64,
        contiguous); returns (Xout, sigout, result)."""
        ctx = self._ctx
        Xout = torch.empty_like(Xv) if Xout is None else Xout
        sigout = torch.empty_like(sigv) if sigout is None else sigout
        res = nat.StepResult()
        while True:
            p = self.params()
            nbytes = ctx.lib.ves_biem_step_workspace(ctx.handle, ctypes.byref(p), self.nv)
            w = ws if ws is not None and ws.numel() >= nbytes else ctx.workspace(nbytes)
            rc = ctx.lib.ves_biem_step(ctx.handle, ctypes.byref(p), self.nv, Xv.data_ptr(), sigv.data_ptr(),
                                       Xout.data_ptr(), sigout.data_ptr(), ctypes.byref(res), w.data_ptr(),
                                       w.numel(), nat.stream_ptr(self.device))
            if rc == nat.VES_ERR_NEARLIST_OVERFLOW and self._grow(res):
                continue  # the near lists are built before the solve reads them: re-run with room
            break
        if rc not in (nat.VES_OK, nat.VES_ERR_GMRES_MAXIT):
            nat.check(rc, "time_step")
        self.last = res
        return Xout, sigout, res

    def _grow(self, res) -> bool:
        """After VES_ERR_NEARLIST_OVERFLOW: enlarge the capacity that ran out
        (False if neither did, i.e. the overflow is not a capacity)."""
        need = self._ctx.max_candidates()
        if need > self._maxc:
            self._maxc = nat.grow_capacity(need, self._maxc)
            return True
        maxe = self._maxe if self._maxe > 0 else max(1024, self.nv * self.N)
        if self.near == "matlab" and res.n_near_entries > maxe:
            self._maxe = nat.grow_capacity(res.n_near_entries, maxe)
            return True
        return False

    def time_step(self, Xstore, sigStore, etaStore=None, RSstore=None):
        """tstep_biem.py:181-428 -> (X, sigma, eta, RS, iter, iflag).

        ``iter`` follows the reference's count of time_matvec calls, which
        includes the one call scipy's LinearOperator makes on a zero vector to
        infer its dtype (tstep_biem.py:366); the device solver makes no such
        call, so ``iter = matvecs + 1``.  ``self.last.matvecs`` holds the
        number of operator applications actually performed."""
        X = as_device_f64(Xstore, self.device)
        sig = as_device_f64(sigStore, self.device)
        Xv, sv = to_vm(X), to_vm(sig)
        Xo, so, res = self.step_device(Xv, sv)
        return from_vm(Xo), from_vm(so), None, None, res.matvecs + 1, res.info != 0

    def bg_flow(self, X, Xwalls=None, *args, **kwargs):
        """tstep_biem.py:849-952 for the unconfined flows."""
        X = as_device_f64(X, self.device)
        kind = next((a for a in args if a in nat.FLOW), self.options.get("farField", "shear"))
        if kind not in nat.FLOW:
            raise ValueError("Unknown or missing flow type in bg_flow.")
        speed = float(kwargs.get("Speed", 1.0))
        Xv = to_vm(X)
        out = torch.empty_like(Xv)
        ctx = self._ctx
        nat.check(ctx.lib.ves_bg_flow(ctx.handle, self.nv if X.shape[1] == self.nv else X.shape[1], nat.FLOW[kind],
                                      speed, float(kwargs.get("chanWidth", 1.0)), float(kwargs.get("vortexSize", 1.0)),
                                      Xv.data_ptr(), out.data_ptr(), nat.stream_ptr(self.device)), "bg_flow")
        return from_vm(out)


class TStepBiemMixed:
    """One implicit step of a suspension of several point counts.

    ``Xs`` is a list of groups, each an X[2N_g, nv_g] array in the reference
    layout (the reference itself holds one N per suspension; this class has
    no counterpart there).  Every vesicle of every group is in one GMRES
    system.  Within a group the step is TStepBiem's with the given ``near``
    rule; between groups the far field runs over the source group's
    upsampled points and the near zone and its correction follow the MATLAB
    rules with a separate target set (getZone's NearOther and nearSingInt
    with tEqualS false, matlab/capsules_py.m:194-467,
    matlab/poten_py.m:495-692), h = the source group's min length / N.
    ``near`` is "matlab" or "none"; no viscosity contrast, repulsion or walls.
    """

    def __init__(self, Xs, options, prams, near: str = "matlab", farfield_precision: str = "fp32c",
                 sl_precision: str = "fp32c", device=None, precond_precision: str = "fp64"):
        if near not in ("matlab", "none"):
            raise NotImplementedError("TStepBiemMixed: near must be 'matlab' or 'none'")
        if not 1 <= len(Xs) <= 4:
            raise ValueError("TStepBiemMixed: 1 to 4 groups")
        if options.get("repulsion", False):
            raise NotImplementedError("TStepBiemMixed: no repulsion between groups")
        self.groups = [TStepBiem(X, None, options, prams, near=near, farfield_precision=farfield_precision,
                                 sl_precision=sl_precision, device=device, precond_precision=precond_precision)
                       for X in Xs]
        if any(g._visc is not None for g in self.groups):
            raise NotImplementedError("TStepBiemMixed: no viscosity contrast")
        if any(g.nv < 1 for g in self.groups):
            raise ValueError("TStepBiemMixed: every group needs a vesicle")
        self.device = self.groups[0].device
        self.last = None

    def _arrays(self):
        ng = len(self.groups)
        ctxs = (ctypes.c_void_p * ng)(*[g._ctx.handle for g in self.groups])
        nvs = (ctypes.c_int * ng)(*[g.nv for g in self.groups])
        return ng, ctxs, nvs

    def workspace_bytes(self) -> int:
        ng, ctxs, nvs = self._arrays()
        p = self.groups[0].params()
        lib = self.groups[0]._ctx.lib
        return int(lib.ves_biem_step_mixed_workspace(ng, ctypes.cast(ctxs, ctypes.c_void_p), ctypes.byref(p),
                                                     ctypes.cast(nvs, ctypes.c_void_p)))

    def time_step(self, Xs, sigs):
        """-> (list of X, list of sigma, iter, iflag); ``iter`` counts the
        operator applications plus one, as TStepBiem.time_step."""
        ng, ctxs, nvs = self._arrays()
        p = self.groups[0].params()
        lib = self.groups[0]._ctx.lib
        Xv = [to_vm(as_device_f64(X, self.device)) for X in Xs]
        sv = [to_vm(as_device_f64(s, self.device)) for s in sigs]
        for g, X, sg in zip(self.groups, Xv, sv):
            if X.shape != (g.nv, 2 * g.N) or sg.shape != (g.nv, g.N):
                raise ValueError("TStepBiemMixed.time_step: group shapes changed")
        Xo = [torch.empty_like(X) for X in Xv]
        so = [torch.empty_like(s) for s in sv]

        def ptrs(ts):
            return ctypes.cast((ctypes.c_void_p * ng)(*[t.data_ptr() for t in ts]), ctypes.c_void_p)

        res = nat.StepResult()
        while True:
            p = self.groups[0].params()
            nbytes = self.workspace_bytes()
            if nbytes == 0:
                nat.check(nat.VES_ERR_ARG, "time_step (mixed): workspace query")
            ws = self.groups[0]._ctx.workspace(nbytes)
            rc = lib.ves_biem_step_mixed(ng, ctypes.cast(ctxs, ctypes.c_void_p), ctypes.byref(p),
                                         ctypes.cast(nvs, ctypes.c_void_p), ptrs(Xv), ptrs(sv), ptrs(Xo), ptrs(so),
                                         ctypes.byref(res), ws.data_ptr(), ws.numel(), nat.stream_ptr(self.device))
            if rc == nat.VES_ERR_NEARLIST_OVERFLOW:
                need = max(g._ctx.max_candidates() for g in self.groups)
                g0 = self.groups[0]
                if need > g0._maxc:
                    for g in self.groups:
                        g._maxc = nat.grow_capacity(need, g0._maxc)
                    continue
                maxe = g0._maxe if g0._maxe > 0 else max(1024, max(g.nv * g.N for g in self.groups))
                if res.n_near_entries > maxe:
                    for g in self.groups:
                        g._maxe = nat.grow_capacity(res.n_near_entries, maxe)
                    continue
            break
        if rc not in (nat.VES_OK, nat.VES_ERR_GMRES_MAXIT):
            nat.check(rc, "time_step (mixed)")
        self.last = res
        return [from_vm(X) for X in Xo], [from_vm(s) for s in so], res.matvecs + 1, res.info != 0
