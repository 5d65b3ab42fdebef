"""MLARM surrogate step on the device (newtorch/wrapper_MLARM_batch_compile_N128.py).

``MLARM_manyfree_py`` keeps the reference constructor and
``time_step_many_noinfo(Xold, tenOld, nlayers)`` signature.  The five
networks are loaded from the same TorchScript files the reference loads
(``../trained/torch_script_models/*.pt`` relative to the working directory,
``:671-707``) unless state dicts are passed; their weights move once to the
device engine of ``ves_nets.cu``.  A step is one call of ``ves_mlarm_step``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np
import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, to_vm
from .mlarm_weights import MODEL_FILES, NETS

_ORDER = ("conv1_1.weight", "conv1_1.bias", "conv1_2.weight", "conv1_2.bias", "conv2_1.weight", "conv2_1.bias",
          "conv2_2.weight", "conv2_2.bias", "deconv1.weight", "deconv1.bias", "deconv2.weight", "deconv2.bias",
          "mix.weight", "mix.bias",
          "bn1.weight", "bn1.bias", "bn1.running_mean", "bn1.running_var",
          "bn2.weight", "bn2.bias", "bn2.running_mean", "bn2.running_var",
          "bn3.weight", "bn3.bias", "bn3.running_mean", "bn3.running_var",
          "bn4.weight", "bn4.bias", "bn4.running_mean", "bn4.running_var")


def load_state_dict(path: str):
    """Parameters of a TorchScript model file as float32 numpy arrays."""
    m = torch.jit.load(path, map_location="cpu")
    return {k: v.detach().cpu().numpy().astype(np.float32) for k, v in m.state_dict().items()}


class Network:
    """One network on the device (``ves_net``), built from a state dict in the
    reference's parameter naming.  ``autotune`` (BF16 tensor-core networks):
    the first forward pass at each vesicle count times the launch shapes of
    every block and keeps the fastest (ves_net_set_autotune)."""

    def __init__(self, name: str, state_dict, precision: str = "fp32", device=None, autotune: bool = True):
        self.name = name
        self.spec = NETS[name]
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        lib = nat.load_library()
        self.lib = lib
        blocks = (nat.NetBlock * len(self.spec.blocks))()
        arrays = []
        for i, b in enumerate(self.spec.blocks):
            blocks[i] = nat.NetBlock(b.cin, b.c1, b.c2, b.cmix, int(b.residual), b.npass)
            for key in _ORDER:
                a = state_dict[f"{b.prefix}.{key}"]
                a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
                arrays.append(np.ascontiguousarray(a, dtype=np.float32))
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            nat.check(lib.ves_net_create(nat.NET_PREC[precision], self.spec.rep, self.spec.L, len(self.spec.blocks),
                                         blocks, ptrs, ctypes.byref(h)), f"ves_net_create({name})")
        self.handle = h
        self._ws = None
        if autotune and precision == "bf16":
            nat.check(lib.ves_net_set_autotune(h, 1), f"ves_net_set_autotune({name})")

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        """model(x) for x of shape (nv, rep*cin, L) on the device."""
        x = x.to(self.device, self.dtype).contiguous()
        nv = x.shape[0]
        out = torch.empty((nv, self.spec.rep * self.spec.cout, self.spec.L), dtype=self.dtype, device=self.device)
        need = self.lib.ves_net_forward_workspace(self.handle, nv)
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        nat.check(self.lib.ves_net_forward(self.handle, nv, x.data_ptr(), out.data_ptr(), self._ws.data_ptr(),
                                           self._ws.numel(), nat.stream_ptr(self.device)), f"net {self.name}")
        return out

    __call__ = forward

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.ves_net_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


def _f64(a):
    return np.ascontiguousarray(np.asarray(a.detach().cpu() if isinstance(a, torch.Tensor) else a, dtype=np.float64))


class MLARM_manyfree_py:
    """MLARM_manyfree_py (wrapper_MLARM_batch_compile_N128.py:649-710) for N = 128.

    Extra keyword arguments: ``state_dicts`` ({name: state dict} for the five
    networks "relax", "adv", "near", "selften", "advten"; default: the
    reference's TorchScript files under ``model_dir``), ``net_precision``
    ("fp32", the reference networks' type, "fp64", or "bf16" on the tensor
    cores), ``farfield_precision``
    ("fp32c" or "fp64"), ``eval_near_net`` (evaluate the near-field
    network as the reference does; its output enters the step only through
    the repulsion force) and ``autotune`` (launch shapes of the BF16 network
    kernels timed on the first step at each vesicle count), ``judge_tol``
    (> 0: the plain BIEM step judges every vesicle's surrogate step and
    replaces it where it moved the vesicle's area or length by more than
    ``judge_tol``, relative: the implicit step of the isolated vesicle with
    the step's explicit velocity; ``last_result.n_fallback`` counts them; 0,
    the default, is the reference's step) and ``conserve`` (the advection and
    relaxation displacements made area- and length-preserving to first order,
    as the exact dynamics is; off: the reference's step) and
    ``area_len_tol`` (the area/length correction's tolerance; 0: the
    reference's 1e-2).
    """

    def __init__(self, dt, vinf, oc, use_repulsion, repStrength, rbf_upsample: int,
                 advNetInputNorm, advNetOutputNorm, relaxNetInputNorm, relaxNetOutputNorm,
                 nearNetInputNorm, nearNetOutputNorm, tenSelfNetInputNorm, tenSelfNetOutputNorm,
                 tenAdvNetInputNorm, tenAdvNetOutputNorm, device, logger=None, *, state_dicts=None,
                 model_dir: str = "../trained/torch_script_models", net_precision: str = "fp32",
                 farfield_precision: str = "fp32c", eval_near_net: bool = True, autotune: bool = True,
                 judge_tol: float = 0.0, conserve: bool = False, area_len_tol: float = 0.0):
        if use_repulsion:
            raise NotImplementedError("MLARM_manyfree_py: repulsion is not supported")
        self.dt = float(dt)
        self.vinf = vinf
        self.oc = oc
        self.kappa = 1.0
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("MLARM_manyfree_py runs on a CUDA device")
        self.logger = logger
        self.use_repulsion = use_repulsion
        self.repStrength = repStrength
        self.rbf_upsample = rbf_upsample
        self.farfield_precision = farfield_precision
        self.eval_near_net = bool(eval_near_net)
        self.judge_tol = float(judge_tol)
        self.conserve = bool(conserve)
        self.area_len_tol = float(area_len_tol)
        self.area0 = None
        self.len0 = None
        self._norms = {
            "adv_in": _f64(advNetInputNorm), "adv_out": _f64(advNetOutputNorm),
            "relax_in": _f64(relaxNetInputNorm), "relax_out": _f64(relaxNetOutputNorm),
            "near_in": _f64(nearNetInputNorm), "near_out": _f64(nearNetOutputNorm),
            "selften_in": _f64(tenSelfNetInputNorm), "selften_out": _f64(tenSelfNetOutputNorm),
            "advten_in": _f64(tenAdvNetInputNorm), "advten_out": _f64(tenAdvNetOutputNorm),
        }
        shapes = {"adv_in": (127, 4), "adv_out": (127, 4), "relax_in": (4,), "relax_out": (4,),
                  "near_in": (128, 4), "near_out": (128, 2, 12), "selften_in": (4,), "selften_out": (2,),
                  "advten_in": (127, 4), "advten_out": (127, 4)}
        for k, shp in shapes.items():
            if self._norms[k].shape != shp:
                raise ValueError(f"MLARM_manyfree_py: {k} has shape {self._norms[k].shape}, expected {shp}")
        if state_dicts is None:
            state_dicts = {n: load_state_dict(os.path.join(model_dir, MODEL_FILES[n])) for n in NETS}
        with torch.cuda.device(self.device):
            self.nets = {n: Network(n, state_dicts[n], net_precision, self.device, autotune=autotune) for n in NETS}
        self.ctx = nat.context(128, self.device)
        lib = self.ctx.lib
        self.lib = lib
        nr = nat.MlarmNorms(*[self._norms[k].ctypes.data for k in
                              ("adv_in", "adv_out", "relax_in", "relax_out", "near_in", "near_out", "selften_in",
                               "selften_out", "advten_in", "advten_out")])
        h = ctypes.c_void_p()
        n = self.nets
        nat.check(lib.ves_mlarm_create(self.ctx.handle, n["relax"].handle, n["adv"].handle, n["near"].handle,
                                       n["selften"].handle, n["advten"].handle, ctypes.byref(nr), ctypes.byref(h)),
                  "ves_mlarm_create")
        self.handle = h
        self.last_result = None
        # near-pair candidate capacity per vesicle; grows (and the step is
        # re-run from its unchanged inputs) when a step reports more candidates
        self._maxc = 32

    def _params(self):
        return nat.MlarmParams(self.dt, self.kappa, nat.FLOW["shear"], 0.0, 0.0, 0.0,
                               nat.PREC[self.farfield_precision], 1 if self.eval_near_net else 0, self._maxc,
                               self.judge_tol, 1 if self.conserve else 0, self.area_len_tol)

    def _step(self, Xold, tenOld, trace=None):
        X = as_device_f64(Xold, self.device)
        N, nv = X.shape[0] // 2, X.shape[1]
        if N != 128:
            raise ValueError("MLARM_manyfree_py: the networks are built for N = 128 (got %d)" % N)
        if self.area0 is None or self.len0 is None:
            raise ValueError("MLARM_manyfree_py: set area0 and len0 before stepping (entry driver :157-161)")
        Xv = to_vm(X)
        tv = to_vm(as_device_f64(tenOld, self.device))
        vb = to_vm(as_device_f64(self.vinf(X), self.device))
        a0 = as_device_f64(self.area0, self.device).reshape(-1).contiguous()
        l0 = as_device_f64(self.len0, self.device).reshape(-1).contiguous()
        Xo = torch.empty_like(Xv)
        to = torch.empty_like(tv)
        res = nat.MlarmResult()
        tr = ctypes.byref(trace) if trace is not None else None
        while True:
            prm = self._params()
            ws = self.ctx.workspace(self.lib.ves_mlarm_step_workspace(self.handle, ctypes.byref(prm), nv))
            rc = self.lib.ves_mlarm_step(self.handle, ctypes.byref(prm), nv, Xv.data_ptr(), tv.data_ptr(),
                                         vb.data_ptr(), a0.data_ptr(), l0.data_ptr(), Xo.data_ptr(), to.data_ptr(),
                                         ctypes.byref(res), tr, ws.data_ptr(), ws.numel(), nat.stream_ptr(self.device))
            need = self.ctx.max_candidates()
            if rc == nat.VES_ERR_NEARLIST_OVERFLOW and need > self._maxc:
                # the lists are built before anything reads them: grow and re-run
                self._maxc = nat.grow_capacity(need, self._maxc)
                continue
            nat.check(rc, "ves_mlarm_step")
            break
        self.last_result = res
        return from_vm(Xo), from_vm(to)

    def time_step_many_noinfo(self, Xold, tenOld, nlayers: int = 3):
        """One MLARM step (:986-1206): returns (Xnew [2N, nv], tenNew [N, nv])."""
        if nlayers != 3:
            raise NotImplementedError("MLARM_manyfree_py: nlayers = 3 only (the N = 128 near network)")
        return self._step(Xold, tenOld)

    def time_step_trace(self, Xold, tenOld):
        """time_step_many_noinfo plus its stage outputs (reference layouts)."""
        X = as_device_f64(Xold, self.device)
        N, nv = X.shape[0] // 2, X.shape[1]
        f64 = dict(dtype=torch.float64, device=self.device)
        buf = {
            "Xstand": torch.empty(nv, 2 * N, **f64), "scaling": torch.empty(nv, **f64),
            "rotate": torch.empty(nv, **f64), "rot_center": torch.empty(nv, 2, **f64),
            "trans": torch.empty(nv, 2, **f64), "sort_idx": torch.empty(nv, N, dtype=torch.int32, device=self.device),
            "far1": torch.empty(nv, 2 * N, **f64), "far2": torch.empty(nv, 2 * N, **f64),
            "vback_solve": torch.empty(nv, N, **f64), "selfbend_solve": torch.empty(nv, N, **f64),
            "Xadv": torch.empty(nv, 2 * N, **f64), "Xrelax": torch.empty(nv, 2 * N, **f64),
            "Xalign": torch.empty(nv, 2 * N, **f64), "Xcorr": torch.empty(nv, 2 * N, **f64),
        }
        tr = nat.MlarmTrace(*[buf[k].data_ptr() for k in ("Xstand", "scaling", "rotate", "rot_center", "trans",
                                                          "sort_idx", "far1", "far2", "vback_solve",
                                                          "selfbend_solve", "Xadv", "Xrelax", "Xalign", "Xcorr")])
        Xn, tn = self._step(Xold, tenOld, tr)
        out = {"X": Xn, "ten": tn}
        for k, v in buf.items():
            if k in ("scaling", "rotate"):
                out[k] = v
            elif k in ("rot_center", "trans"):
                out[k] = v.t().contiguous()
            elif k == "sort_idx":
                out[k] = v
            else:
                out[k] = from_vm(v)
        return out

    def standardizationStep(self, Xin):
        """standardizationStep (:4119-4138): (Xstand, (scaling, rotate, rotCenter, trans, sortIdx))."""
        X = as_device_f64(Xin, self.device)
        N, nv = X.shape[0] // 2, X.shape[1]
        f64 = dict(dtype=torch.float64, device=self.device)
        Xs = torch.empty(nv, 2 * N, **f64)
        sc, rot = torch.empty(nv, **f64), torch.empty(nv, **f64)
        rc, tr = torch.empty(nv, 2, **f64), torch.empty(nv, 2, **f64)
        si = torch.empty(nv, N, dtype=torch.int32, device=self.device)
        ws = self.ctx.workspace(self.lib.ves_mlarm_standardize_workspace(self.ctx.handle, nv))
        nat.check(self.lib.ves_mlarm_standardize(self.ctx.handle, nv, to_vm(X).data_ptr(), Xs.data_ptr(),
                                                 sc.data_ptr(), rot.data_ptr(), rc.data_ptr(), tr.data_ptr(),
                                                 si.data_ptr(), ws.data_ptr(), ws.numel(),
                                                 nat.stream_ptr(self.device)), "standardizationStep")
        return from_vm(Xs), (sc, rot, rc.t().contiguous(), tr.t().contiguous(), si.long())

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.ves_mlarm_destroy(self.handle)
                self.handle = None
        except Exception:
            pass
