"""ctypes binding of the C-ABI library ``_lib/libves2d_gb300.so``.

The library is the only compute path of this package: every operator below
calls one of its ``extern "C"`` entry points on device memory owned by
PyTorch.  If the library is missing, importing an operator raises; there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libves2d_gb300.so")

VES_OK = 0
VES_ERR_SHAPE = 1
VES_ERR_NONFINITE = 2
VES_ERR_NEARLIST_OVERFLOW = 3
VES_ERR_GMRES_MAXIT = 4
VES_ERR_CUDA = 5
VES_ERR_ARG = 6
VES_ERR_TIMEOUT = 7
VES_ERR_SINGULAR = 8
VES_ERR_WORKSPACE = 9

PREC = {"fp64": 0, "fp32c": 1, "fp32m": 2}
NEAR = {"none": 0, "py_hh": 1, "matlab": 2, "py_rbf": 3}
FLOW = {"relaxation": 0, "extensional": 1, "parabolic": 2, "taylorGreen": 3, "shear": 4, "vortex": 5}


class VesError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class NearListOverflow(VesError):
    pass


class GmresNotConverged(VesError):
    pass


class NearLists(ctypes.Structure):
    _fields_ = [
        ("maxc", ctypes.c_int),
        ("cand_count", ctypes.c_void_p),
        ("cand_src", ctypes.c_void_p),
        ("excl_mask", ctypes.c_void_p),
        ("hh_mask", ctypes.c_void_p),
        ("max_entries", ctypes.c_int),
        ("n_entries", ctypes.c_void_p),
        ("ent_tsj", ctypes.c_void_p),
        ("ent_icp", ctypes.c_void_p),
        ("ent_geo", ctypes.c_void_p),
    ]


class StepParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("gmres_tol", ctypes.c_double),
        ("gmres_maxiter", ctypes.c_int),
        ("gmres_restart", ctypes.c_int),
        ("use_preco", ctypes.c_int),
        ("flow", ctypes.c_int),
        ("speed", ctypes.c_double),
        ("chan_width", ctypes.c_double),
        ("vortex_size", ctypes.c_double),
        ("near_scheme", ctypes.c_int),
        ("farfield_precision", ctypes.c_int),
        ("sl_precision", ctypes.c_int),
        ("maxc", ctypes.c_int),
        ("max_entries", ctypes.c_int),
        ("repulsion", ctypes.c_int),
        ("rep_strength", ctypes.c_double),
        ("min_dist", ctypes.c_double),
        ("visc_cont", ctypes.c_void_p),
    ]


class StepResult(ctypes.Structure):
    _fields_ = [
        ("matvecs", ctypes.c_int),
        ("inner_iters", ctypes.c_int),
        ("info", ctypes.c_int),
        ("resid", ctypes.c_double),
        ("n_near_pairs", ctypes.c_int),
        ("n_near_entries", ctypes.c_int),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("kernel_launches", ctypes.c_longlong),
        ("farfield_launches", ctypes.c_longlong),
        ("farfield_ms", ctypes.c_double),
        ("farfield_pairs", ctypes.c_double),
        ("farfield_mp_terms", ctypes.c_double),
        ("farfield_direct_pairs", ctypes.c_double),
        ("networks_launches", ctypes.c_longlong),
        ("networks_ms", ctypes.c_double),
        ("networks_flops", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_LL = ctypes.c_longlong
_SZ = ctypes.c_size_t

# name: (restype, argtypes)
class NetBlock(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("cin", "c1", "c2", "cmix", "residual", "npass")]


class MlarmNorms(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("adv_in", "adv_out", "relax_in", "relax_out", "near_in", "near_out",
                                               "selften_in", "selften_out", "advten_in", "advten_out")]


class MlarmParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("flow", ctypes.c_int),
        ("speed", ctypes.c_double),
        ("chan_width", ctypes.c_double),
        ("vortex_size", ctypes.c_double),
        ("farfield_precision", ctypes.c_int),
        ("eval_near_net", ctypes.c_int),
        ("maxc", ctypes.c_int),
        ("judge_tol", ctypes.c_double),
        ("conserve", ctypes.c_int),
        ("area_len_tol", ctypes.c_double),
    ]


class MlarmResult(ctypes.Structure):
    _fields_ = [("n_near_pairs", ctypes.c_int), ("auglag_iters", ctypes.c_int), ("n_fallback", ctypes.c_int)]


class MlarmTrace(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("Xstand", "scaling", "rotate", "rot_center", "trans", "sort_idx",
                                               "far1", "far2", "vback_solve", "selfbend_solve", "Xadv", "Xrelax",
                                               "Xalign", "Xcorr")]


NET_PREC = {"fp64": 0, "fp32": 1, "bf16": 2}

SIGNATURES = {
    "ves_ctx_create": (_I, [_I, ctypes.POINTER(_P)]),
    "ves_ctx_destroy": (_I, [_P]),
    "ves_ctx_info": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "ves_ctx_max_candidates": (_I, [_P]),
    "ves_last_error": (ctypes.c_char_p, []),
    "ves_diff_prop": (_I, [_P, _I, _I, _P, _P, _P, _P, _P]),
    "ves_geom_prop": (_I, [_P, _I, _P, _P, _P, _P, _P]),
    "ves_upsample": (_I, [_P, _I, _I, _P, _P, _P]),
    "ves_trac_jump": (_I, [_P, _I, _D, _P, _P, _P, _LL, _P, _LL, _P, _P]),
    "ves_surface_div": (_I, [_P, _I, _P, _P, _P, _LL, _P, _LL, _P]),
    "ves_compute_derivs": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "ves_compute_derivs_workspace": (_SZ, [_P, _I]),
    "ves_bg_flow": (_I, [_P, _I, _I, _D, _D, _D, _P, _P, _P]),
    "ves_stokes_sl_matrix": (_I, [_P, _I, _P, _I, _P, _P, _SZ, _P]),
    "ves_stokes_sl_matrix_workspace": (_SZ, [_P, _I, _I]),
    "ves_sl_diag": (_I, [_I, _I, _P, _P, _P, _P]),
    "ves_near_zone_py": (_I, [_P, _I, _P, _P, _D, ctypes.POINTER(NearLists), _P, _SZ, _P]),
    "ves_near_zone_matlab": (_I, [_P, _I, _P, _D, ctypes.POINTER(NearLists), _P, _SZ, _P]),
    "ves_near_zone_workspace": (_SZ, [_P, _I]),
    "ves_farfield": (_I, [_P, _I, _I, _I, _P, _P, _I, _I, _P, _P, ctypes.POINTER(NearLists), _P, _P, _SZ, _P]),
    "ves_farfield_workspace": (_SZ, [_P, _I, _I, _I, _I, _I]),
    "ves_density": (_I, [_I, _I, _P, _P, _P, _P]),
    "ves_near_sing_int": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, ctypes.POINTER(NearLists), _D, _P, _P, _P,
                               _SZ, _P]),
    "ves_near_sing_int_workspace": (_SZ, [_P, _I, _I]),
    "ves_biem_step": (_I, [_P, ctypes.POINTER(StepParams), _I, _P, _P, _P, _P, ctypes.POINTER(StepResult), _P,
                           _SZ, _P]),
    "ves_biem_step_workspace": (_SZ, [_P, ctypes.POINTER(StepParams), _I]),
    "ves_biem_step_mixed": (_I, [_I, _P, ctypes.POINTER(StepParams), _P, _P, _P, _P, _P,
                                 ctypes.POINTER(StepResult), _P, _SZ, _P]),
    "ves_biem_step_mixed_workspace": (_SZ, [_I, _P, ctypes.POINTER(StepParams), _P]),
    "ves_redistribute_arclength": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(_I), _P, _SZ, _P]),
    "ves_redistribute_arclength_workspace": (_SZ, [_P, _I]),
    "ves_net_set_autotune": (_I, [_P, _I]),
    "ves_net_create": (_I, [_I, _I, _I, _I, ctypes.POINTER(NetBlock), ctypes.POINTER(ctypes.c_void_p),
                            ctypes.POINTER(_P)]),
    "ves_net_destroy": (_I, [_P]),
    "ves_net_info": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                          ctypes.POINTER(_I)]),
    "ves_net_forward": (_I, [_P, _I, _P, _P, _P, _SZ, _P]),
    "ves_net_forward_workspace": (_SZ, [_P, _I]),
    "ves_mlarm_create": (_I, [_P, _P, _P, _P, _P, _P, ctypes.POINTER(MlarmNorms), ctypes.POINTER(_P)]),
    "ves_mlarm_destroy": (_I, [_P]),
    "ves_mlarm_step": (_I, [_P, ctypes.POINTER(MlarmParams), _I, _P, _P, _P, _P, _P, _P, _P,
                            ctypes.POINTER(MlarmResult), ctypes.POINTER(MlarmTrace), _P, _SZ, _P]),
    "ves_mlarm_step_workspace": (_SZ, [_P, ctypes.POINTER(MlarmParams), _I]),
    "ves_mlarm_standardize": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "ves_mlarm_standardize_workspace": (_SZ, [_P, _I]),
    "ves_align_center_angle": (_I, [_P, _I, _P, _P, _P, _P]),
    "ves_center_angle": (_I, [_P, _I, _P, _P, _P, _P]),
    "ves_correct_area_length": (_I, [_P, _I, _P, _P, _P, _P, ctypes.POINTER(_I), _P, _SZ, _P]),
    "ves_correct_area_length_workspace": (_SZ, [_P, _I]),
    "ves_farfield_static_scratch": (_I, [_I, _I, _I, _P, _P, _I, _I, _P, _P, _P, _P]),
    "ves_ctx_set_timing": (_I, [_P, _I]),
    "ves_ctx_stats": (_I, [_P, ctypes.POINTER(Stats), _I]),
    "ves_probe_sfu_peak": (_I, [ctypes.POINTER(ctypes.c_double), _P]),
    "ves_upsample_geometry": (_I, [_P, _I, _P, _P, _P, _P, _P, _P]),
    "ves_probe_wait_timeout": (_I, [_P, _P]),
    "ves_stokes_dl_matrix": (_I, [_P, _I, _P, _P, _I, _P, _P, _SZ, _P]),
    "ves_stokes_dl_matrix_workspace": (_SZ, [_P, _I, _I]),
    "ves_dl_density": (_I, [_I, _I, _P, _P, _P, _P, _P]),
    "ves_farfield_dl": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _I, _I, _P, _P, ctypes.POINTER(NearLists), _P,
                             _P, _SZ, _P]),
    "ves_farfield_dl_workspace": (_SZ, [_I, _I, _I, _I]),
    "ves_near_sing_int_dl": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, ctypes.POINTER(NearLists), _D, _P,
                                  _P, _P, _SZ, _P]),
    "ves_near_sing_int_dl_workspace": (_SZ, [_P, _I]),
    "ves_repulsion_force_workspace": (_SZ, [_I]),
    "ves_repulsion_force": (_I, [_I, _I, _P, _D, _D, _P, _P, _SZ, _P]),
    "ves_traj_create": (_I, [ctypes.c_char_p, _I, _I, _P, _I, _I, ctypes.POINTER(_P)]),
    "ves_traj_append": (_I, [_P, _D, _P, _I, _P]),
    "ves_traj_flush": (_I, [_P, ctypes.POINTER(_LL)]),
    "ves_traj_close": (_I, [_P]),
    "ves_mlarm_targets": (_I, [_P, _I, _P, ctypes.c_double, ctypes.c_double, _I, _P, _P, _P, _P, _P, _SZ, _P]),
    "ves_mlarm_targets_workspace": (_SZ, [_P, _I, _I]),
    "ves_isolated_step": (_I, [_P, _I, _P, _P, ctypes.c_double, ctypes.c_double, _I, _P, _P, _SZ, _P]),
    "ves_isolated_step_workspace": (_SZ, [_P, _I, _I]),
    "ves_trainer_create": (_I, [_I, _I, _I, _P, _P, _I, ctypes.POINTER(_P)]),
    "ves_trainer_destroy": (_I, [_P]),
    "ves_trainer_num_params": (ctypes.c_longlong, [_P]),
    "ves_trainer_forward": (_I, [_P, _I, _P, _P, _P]),
    "ves_trainer_backward_mse": (_I, [_P, _I, _P, _P, _P, ctypes.POINTER(ctypes.c_double), _P]),
    "ves_trainer_adam": (_I, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _I, _P]),
    "ves_trainer_get_params": (_I, [_P, _P, _P]),
    "ves_trainer_get_grads": (_I, [_P, _P, _P]),
    "ves_trainer_get_grads_f64": (_I, [_P, _P, _P]),
}

_lib = None
_lock = threading.Lock()


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the C-ABI library and bind every declared entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError(
                f"ves2dpy_gb300: native library {path} is missing; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return load_library().ves_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc == VES_OK:
        return
    msg = f"{what}: {last_error()}" if what else last_error()
    if rc == VES_ERR_NONFINITE:
        raise ValueError("NaN or Inf in the logpart (" + msg + ")")
    if rc == VES_ERR_NEARLIST_OVERFLOW:
        raise NearListOverflow(rc, msg)
    if rc == VES_ERR_GMRES_MAXIT:
        raise GmresNotConverged(rc, msg)
    if rc in (VES_ERR_SHAPE, VES_ERR_ARG):
        raise ValueError(msg)
    raise VesError(rc, msg)


def grow_capacity(need: int, floor: int = 16) -> int:
    """A list capacity for ``need`` entries with room to spare: the next power
    of two at or above 1.25 x need (at least ``floor``)."""
    c = max(int(floor), 1)
    while c < 1.25 * need:
        c *= 2
    return c


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class Context:
    """One ves_ctx (per-N tables) on one CUDA device, plus a grow-only
    workspace tensor reused by every call on this context."""

    def __init__(self, N: int, device: torch.device):
        self.lib = load_library()
        self.N = int(N)
        self.device = torch.device(device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.ves_ctx_create(self.N, ctypes.byref(h)), "ves_ctx_create")
        self.handle = h
        n, nup, nq = _I(), _I(), _I()
        check(self.lib.ves_ctx_info(h, ctypes.byref(n), ctypes.byref(nup), ctypes.byref(nq)))
        self.Nup = nup.value
        self.nquad = nq.value
        self._ws = None

    def max_candidates(self) -> int:
        """Largest near-pair candidate count of the last call's near-zone builds."""
        return int(self.lib.ves_ctx_max_candidates(self.handle))

    def set_timing(self, on: bool) -> None:
        check(self.lib.ves_ctx_set_timing(self.handle, 1 if on else 0), "set_timing")

    def stats(self, reset: bool = False) -> Stats:
        st = Stats()
        check(self.lib.ves_ctx_stats(self.handle, ctypes.byref(st), 1 if reset else 0), "stats")
        return st

    def workspace(self, nbytes: int) -> torch.Tensor:
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=self.device)
        return self._ws

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.lib is not None:
                self.lib.ves_ctx_destroy(self.handle)
        except Exception:
            pass


_contexts: dict = {}


def probe_sfu_peak(device=None) -> float:
    """Measured MUFU (lg2 + rcp) operations per second of the current GPU."""
    lib = load_library()
    v = ctypes.c_double()
    check(lib.ves_probe_sfu_peak(ctypes.byref(v), stream_ptr(device)), "probe_sfu_peak")
    return v.value


def context(N: int, device) -> Context:
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("ves2dpy_gb300 runs on CUDA devices only (got %s)" % device)
    idx = device.index if device.index is not None else torch.cuda.current_device()
    key = (int(N), idx)
    ctx = _contexts.get(key)
    if ctx is None:
        ctx = Context(N, torch.device("cuda", idx))
        _contexts[key] = ctx
    return ctx
