"""Training the MLARM networks on data that the BIEM operators generate.

The reference loads trained TorchScript models and normalisation constants
(newtorch/entry_driver_manyfreeSpaceVesicle_N128.py:120-145,
wrapper_MLARM_batch_compile_N128.py:650-710) whose weights, data and
training code are not part of its tree.  This module makes them on the GPU:

* shapes: perturbed ellipses of the benchmark's generator over a range of
  reduced areas, evolved by the implicit step of non-interacting vesicles in
  shear flow and at rest (``ves_isolated_step``), then standardised as the
  step standardises them (``ves_mlarm_standardize``);
* targets: what the plain BIEM operators of each vesicle give
  (``ves_mlarm_targets``): the relaxation displacement over one step, the
  self-bending tension, and the tension and velocity responses to the Fourier
  basis velocities;
* training: one channel group of each network with the device trainer
  (``ves_trainer``: forward, backward of every layer type, Adam), then the
  group's weights in every group of the merged network.

The merged networks hold one group per Fourier mode (get_network_torch.py
:99-128, one separately trained model per mode).  Here the advection network
shares one set of weights over the modes (its second input channel is the
mode's basis function, which tells the groups apart), and the
advection-tension network, whose input is the shape alone, tells the modes
apart by a per-mode offset folded into its input normalisation.  Only modes
1-16 and 112-127 (|k| <= 16) are trained: the step filters the interaction
velocity and the new shape to 16 modes (filterShape(., 16), :1094, :1163,
:1198), so a linear background flow has no content in the others; their
output scales are zero, which makes their contribution exactly zero.
"""
from __future__ import annotations

import ctypes
import math
import os
import time

import numpy as np
import torch

from . import _native as nat
from .mlarm_weights import NETS, NetSpec, param_shapes

PKG = os.path.dirname(os.path.abspath(__file__))
TRAINED_DIR = os.path.join(PKG, "trained")
N = 128
MODES = 127
NYQUIST = 63                      # rep index of the Nyquist mode (zeroed by the step)
TRAIN_MODES = tuple(list(range(16)) + list(range(111, 127)))   # Fourier index k = kk + 1, |k| <= 16
ORDER = ("conv1_1.weight", "conv1_1.bias", "conv1_2.weight", "conv1_2.bias", "conv2_1.weight", "conv2_1.bias",
         "conv2_2.weight", "conv2_2.bias", "deconv1.weight", "deconv1.bias", "deconv2.weight", "deconv2.bias",
         "mix.weight", "mix.bias",
         "bn1.weight", "bn1.bias", "bn1.running_mean", "bn1.running_var",
         "bn2.weight", "bn2.bias", "bn2.running_mean", "bn2.running_var",
         "bn3.weight", "bn3.bias", "bn3.running_mean", "bn3.running_var",
         "bn4.weight", "bn4.bias", "bn4.running_mean", "bn4.running_var")


def group_spec(name: str) -> NetSpec:
    """The one-group network whose weights fill every group of ``name``."""
    s = NETS[name]
    return NetSpec(name, 1, s.L, s.blocks)


def init_state_dict(spec: NetSpec, seed: int = 0):
    """Initial weights of a one-group network: uniform(+-1/sqrt(fan_in)) for
    convolutions (PyTorch's default scale), the mixing convolution of residual
    blocks scaled by 0.1 (each block starts close to the identity), batch norm
    as the identity map."""
    rng = np.random.default_rng(seed)
    sd = {}
    for name, shape, fan in param_shapes(spec):
        if fan == 0:
            field = name.rsplit(".", 1)[1]
            v = np.ones(shape) if field in ("weight", "running_var") else np.zeros(shape)
        else:
            v = rng.uniform(-1.0, 1.0, size=shape) / math.sqrt(fan)
            if ".mix." in name:
                blk = next(b for b in spec.blocks if name.startswith(b.prefix + "."))
                if blk.residual:
                    v *= 0.1
        sd[name] = v.astype(np.float32)
    return sd


def merge_groups(name: str, sd_group) -> dict:
    """State dict of the merged network ``name`` with the one-group weights
    ``sd_group`` in each of its groups (grouped-convolution layout)."""
    G = NETS[name].rep
    out = {}
    for k, v in sd_group.items():
        v = np.asarray(v, dtype=np.float32)
        out[k] = np.ascontiguousarray(np.concatenate([v] * G, axis=0)) if G > 1 else v.copy()
    return out


class Trainer:
    """One channel group of a network in training on the device (ves_trainer)."""

    def __init__(self, spec: NetSpec, state_dict, precision: str = "fp32", max_batch: int = 256, device=None):
        if spec.rep != 1:
            raise ValueError("Trainer: one channel group (spec.rep == 1)")
        self.spec = spec
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.lib = nat.load_library()
        self.max_batch = int(max_batch)
        blocks = (nat.NetBlock * len(spec.blocks))()
        self._shapes = []
        arrays = []
        for i, b in enumerate(spec.blocks):
            blocks[i] = nat.NetBlock(b.cin, b.c1, b.c2, b.cmix, int(b.residual), b.npass)
            for key in ORDER:
                a = np.ascontiguousarray(np.asarray(state_dict[f"{b.prefix}.{key}"], dtype=np.float32))
                arrays.append(a)
                self._shapes.append((f"{b.prefix}.{key}", a.shape))
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            nat.check(self.lib.ves_trainer_create(nat.NET_PREC["fp64" if precision == "fp64" else "fp32"], spec.L,
                                                  len(spec.blocks), blocks, ptrs, self.max_batch, ctypes.byref(h)),
                      "ves_trainer_create")
        self.handle = h
        self.step_count = 0

    @property
    def cin(self):
        return self.spec.blocks[0].cin

    @property
    def cout(self):
        return self.spec.blocks[-1].cout

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        x = x.to(self.device, self.dtype).contiguous()
        B = x.shape[0]
        y = torch.empty((B, self.cout, self.spec.L), dtype=self.dtype, device=self.device)
        nat.check(self.lib.ves_trainer_forward(self.handle, B, x.data_ptr(), y.data_ptr(), nat.stream_ptr(self.device)),
                  "trainer forward")
        return y

    def backward(self, target: torch.Tensor, channel_weights=None, want_loss: bool = True, sample_weights=None):
        """Mean squared error of the last forward pass against ``target``
        (optionally weighted per channel and per sample) and its gradient into
        the parameters; returns the loss (or None)."""
        t = target.to(self.device, self.dtype).contiguous()
        w = None if channel_weights is None else channel_weights.to(self.device, self.dtype).contiguous()
        ws = None if sample_weights is None else sample_weights.to(self.device, self.dtype).contiguous()
        loss = ctypes.c_double()
        nat.check(self.lib.ves_trainer_backward_mse(self.handle, t.shape[0], t.data_ptr(), nat.ptr(w), nat.ptr(ws),
                                                    ctypes.byref(loss) if want_loss else None,
                                                    nat.stream_ptr(self.device)), "trainer backward")
        return loss.value if want_loss else None

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        nat.check(self.lib.ves_trainer_adam(self.handle, lr, beta1, beta2, eps, self.step_count,
                                            nat.stream_ptr(self.device)), "trainer adam")

    def train_step(self, x, target, lr, channel_weights=None, want_loss=False, sample_weights=None):
        self.forward_only(x)
        loss = self.backward(target, channel_weights, want_loss, sample_weights)
        self.adam(lr)
        return loss

    def forward_only(self, x: torch.Tensor):
        x = x.to(self.device, self.dtype).contiguous()
        nat.check(self.lib.ves_trainer_forward(self.handle, x.shape[0], x.data_ptr(), None,
                                               nat.stream_ptr(self.device)), "trainer forward")

    def _out(self, fn):
        arrays = [np.empty(shp, dtype=np.float32) for _, shp in self._shapes]
        ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
        nat.check(fn(self.handle, ptrs, nat.stream_ptr(self.device)), "trainer copy-out")
        return {name: a for (name, _), a in zip(self._shapes, arrays)}

    def state_dict(self):
        return self._out(self.lib.ves_trainer_get_params)

    def grads(self):
        return self._out(self.lib.ves_trainer_get_grads)

    def grads_f64(self) -> np.ndarray:
        n = int(self.lib.ves_trainer_num_params(self.handle))
        out = np.empty(n, dtype=np.float64)
        nat.check(self.lib.ves_trainer_get_grads_f64(self.handle, out.ctypes.data, nat.stream_ptr(self.device)),
                  "trainer grads")
        return out

    def __del__(self):
        try:
            if getattr(self, "handle", None):
                self.lib.ves_trainer_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


# ---------------------------------------------------------------------------
# data on the device

def _ctx(device):
    return nat.context(N, device)


def standardize(Xv: torch.Tensor) -> torch.Tensor:
    """ves_mlarm_standardize of shapes in the device layout [nv][2N] -> [nv][2N]."""
    ctx = _ctx(Xv.device)
    nv = Xv.shape[0]
    f64 = dict(dtype=torch.float64, device=Xv.device)
    Xs = torch.empty(nv, 2 * N, **f64)
    sc, rot = torch.empty(nv, **f64), torch.empty(nv, **f64)
    rc, tr = torch.empty(nv, 2, **f64), torch.empty(nv, 2, **f64)
    si = torch.empty(nv, N, dtype=torch.int32, device=Xv.device)
    ws = ctx.workspace(ctx.lib.ves_mlarm_standardize_workspace(ctx.handle, nv))
    nat.check(ctx.lib.ves_mlarm_standardize(ctx.handle, nv, Xv.contiguous().data_ptr(), Xs.data_ptr(), sc.data_ptr(),
                                            rot.data_ptr(), rc.data_ptr(), tr.data_ptr(), si.data_ptr(), ws.data_ptr(),
                                            ws.numel(), nat.stream_ptr(Xv.device)), "standardize")
    return Xs


def isolated_step(Xv: torch.Tensor, vinf: torch.Tensor | None, dt: float, kappa: float = 1.0,
                  sl_precision: str = "fp32c") -> torch.Tensor:
    """ves_isolated_step: one implicit step of non-interacting vesicles [nv][2N]."""
    ctx = _ctx(Xv.device)
    nv = Xv.shape[0]
    out = torch.empty_like(Xv)
    ws = ctx.workspace(ctx.lib.ves_isolated_step_workspace(ctx.handle, nv, nat.PREC[sl_precision]))
    nat.check(ctx.lib.ves_isolated_step(ctx.handle, nv, Xv.contiguous().data_ptr(), nat.ptr(vinf), float(dt),
                                        float(kappa), nat.PREC[sl_precision], out.data_ptr(), ws.data_ptr(),
                                        ws.numel(), nat.stream_ptr(Xv.device)), "isolated_step")
    return out


def targets(Xs: torch.Tensor, dt: float = 1e-5, kappa: float = 1.0, which=("relax", "selften", "advten", "adv"),
            sl_precision: str = "fp64"):
    """ves_mlarm_targets for standardised shapes Xs[nv][2N] (device): a dict
    of FP64 device tensors relax [nv][2N], selften [nv][N], advten
    [nv][254][N], adv [nv][254][2N]."""
    ctx = _ctx(Xs.device)
    nv = Xs.shape[0]
    f64 = dict(dtype=torch.float64, device=Xs.device)
    out = {}
    if "relax" in which:
        out["relax"] = torch.empty(nv, 2 * N, **f64)
    if "selften" in which:
        out["selften"] = torch.empty(nv, N, **f64)
    if "advten" in which:
        out["advten"] = torch.empty(nv, 2 * MODES, N, **f64)
    if "adv" in which:
        out["adv"] = torch.empty(nv, 2 * MODES, 2 * N, **f64)
    ws = ctx.workspace(ctx.lib.ves_mlarm_targets_workspace(ctx.handle, nv, nat.PREC[sl_precision]))
    nat.check(ctx.lib.ves_mlarm_targets(ctx.handle, nv, Xs.contiguous().data_ptr(), float(dt), float(kappa),
                                        nat.PREC[sl_precision], nat.ptr(out.get("relax")), nat.ptr(out.get("selften")),
                                        nat.ptr(out.get("advten")), nat.ptr(out.get("adv")), ws.data_ptr(),
                                        ws.numel(), nat.stream_ptr(Xs.device)), "mlarm_targets")
    return out


def random_shapes(n: int, seed: int, reduced_area=(0.6, 0.9), amp=(0.0, 0.04)) -> np.ndarray:
    """n perturbed ellipses (the benchmark generator's family, modes 2..8) with
    reduced areas and perturbation amplitudes drawn uniformly, scaled to unit
    length (the length the step's arc-length redistribution assumes); [n][2N]."""
    from .suspension import vesicle_shape
    rng = np.random.default_rng(seed)
    out = np.empty((n, 2 * N))
    k = np.fft.fftfreq(N, 1.0 / N)
    for i in range(n):
        ra = rng.uniform(*reduced_area)
        x, y = vesicle_shape(N, rng, ra, area=math.pi, amp=rng.uniform(*amp))
        dx = np.real(np.fft.ifft(1j * k * np.fft.fft(x)))
        dy = np.real(np.fft.ifft(1j * k * np.fft.fft(y)))
        length = np.sum(np.hypot(dx, dy)) * 2 * math.pi / N
        out[i, :N], out[i, N:] = (x - x.mean()) / length, (y - y.mean()) / length
    return out


# the benchmark generator's family (reduced area 0.65, radius perturbation
# modes 2..8 with N(0, 0.02) amplitudes) and its first 2.5e-3 time units of
# relaxation: snapshots at t = 0, 4e-5, 1.4e-4, 5.4e-4 and 2.5e-3
SNAPSHOTS = ((0, 0.0), (2, 2e-5), (5, 2e-5), (10, 4e-5), (20, 1e-4))
REDUCED_AREA = (0.6, 0.72)
AMPLITUDE = (0.0, 0.025)


def shape_dataset(n: int, seed: int, device, snapshots=SNAPSHOTS, shear=(0.0, 4.0),
                  reduced_area=REDUCED_AREA, amp=AMPLITUDE, chunk: int = 4096) -> torch.Tensor:
    """Standardised unit-length training shapes [n][2N] on the device: the
    generated shapes and snapshots of their evolution as isolated vesicles in
    shear flow of a random rate (zero: relaxation) by the implicit BIEM step
    (``snapshots``: (steps, dt) taken one after the other from the previous
    snapshot; the early small steps catch the fast relaxation of the
    perturbation modes that the first steps of a simulation go through)."""
    per = int(math.ceil(n / len(snapshots)))
    gen = torch.Generator(device).manual_seed(seed)
    out = []
    for a in range(0, per, chunk):
        m = min(chunk, per - a)
        X = standardize(torch.tensor(random_shapes(m, seed * 7919 + a, reduced_area, amp), dtype=torch.float64,
                                     device=device))
        rate = torch.empty(m, 1, dtype=torch.float64, device=device).uniform_(*shear, generator=gen)
        part = []
        for steps, dt in snapshots:
            for _ in range(steps):
                vinf = torch.cat([rate * X[:, N:], torch.zeros_like(X[:, :N])], dim=1)
                X = standardize(isolated_step(X, vinf, dt))
            part.append(X.clone())
        out.append(torch.stack(part, 0))
    Xs = torch.cat(out, 1).reshape(-1, 2 * N)
    # drop shapes with a point spacing more than 30% off the mean or a
    # non-finite coordinate (the redistribution keeps good shapes near 1)
    d = torch.hypot(Xs[:, 1:N] - Xs[:, :N - 1], Xs[:, N + 1:] - Xs[:, N:2 * N - 1])
    ok = torch.isfinite(Xs).all(1) & (d.amax(1) < 1.3 * d.mean(1)) & (d.amin(1) > 0.7 * d.mean(1))
    Xs = Xs[ok]
    return Xs[:n].contiguous()


# ---------------------------------------------------------------------------
# normalisation constants (the reference constructor's arrays) and batches

def _stats(a: torch.Tensor):
    return float(a.mean()), float(a.std())


class Dataset:
    """Shapes, targets and normalisation constants for the four trained networks."""

    def __init__(self, Xs: torch.Tensor, dt: float = 1e-5, chunk: int = 1024, keep_modes=TRAIN_MODES):
        self.device = Xs.device
        self.Xs = Xs
        self.n = Xs.shape[0]
        self.dt = dt
        self.modes = torch.tensor(keep_modes, dtype=torch.long, device=self.device)
        nm = len(keep_modes)
        f32 = dict(dtype=torch.float32, device=self.device)
        self.relax = torch.empty(self.n, 2 * N, **f32)
        self.selften = torch.empty(self.n, N, **f32)
        self.advten = torch.empty(self.n, nm, 2, N, **f32)     # (z1 real, z2 imag) per kept mode
        self.adv = torch.empty(self.n, nm, 2, 2 * N, **f32)    # (real, imag) channels, [x ++ y]
        ch = torch.stack([2 * self.modes, 2 * self.modes + 1], 1).reshape(-1)
        for a in range(0, self.n, chunk):
            b = min(self.n, a + chunk)
            t = targets(Xs[a:b], dt)
            self.relax[a:b] = t["relax"].float()
            self.selften[a:b] = t["selften"].float()
            self.advten[a:b] = t["advten"][:, ch].reshape(b - a, nm, 2, N).float()
            self.adv[a:b] = t["adv"][:, ch].reshape(b - a, nm, 2, 2 * N).float()
            del t
        # drop shapes whose targets are far outside the bulk (a shape the
        # evolution broke): per-shape maxima above 20 x their median
        rmax = self.relax.abs().amax(1)
        smax = self.selften.abs().amax(1)
        keep = (torch.isfinite(rmax) & torch.isfinite(smax) & (rmax < 20 * rmax.median()) &
                (smax < 20 * smax.median()) & torch.isfinite(self.adv).all(3).all(2).all(1) &
                torch.isfinite(self.advten).all(3).all(2).all(1))
        if not bool(keep.all()):
            k = torch.nonzero(keep).squeeze(1)
            self.Xs, self.relax, self.selften = Xs[k], self.relax[k], self.selften[k]
            self.advten, self.adv = self.advten[k], self.adv[k]
            self.n = self.Xs.shape[0]
            Xs = self.Xs
        self.dropped = int((~keep).sum())
        X = Xs.float()
        mx, sx = _stats(X[:, :N])
        my, sy = _stats(X[:, N:])
        self.shape_norm = np.array([mx, sx, my, sy])
        self.relax_out = np.array([*_stats(self.relax[:, :N]), *_stats(self.relax[:, N:])])
        self.selften_out = np.array(_stats(self.selften))
        # advection network: shape statistics for every mode; output
        # statistics per kept mode, zero scale elsewhere
        self.adv_in = np.tile(self.shape_norm, (MODES, 1))
        self.adv_out = np.zeros((MODES, 4))
        self.advten_out = np.zeros((MODES, 4))
        for j, kk in enumerate(keep_modes):
            self.adv_out[kk] = [*_stats(self.adv[:, j, 0]), *_stats(self.adv[:, j, 1])]
            self.advten_out[kk] = [*_stats(self.advten[:, j, 0]), *_stats(self.advten[:, j, 1])]
        # advection-tension network: the mode's offset (cx, cy) on a grid is
        # added to the normalised input, mean' = mean - c * std
        self.offsets = np.zeros((MODES, 2))
        g = int(math.ceil(math.sqrt(len(keep_modes))))
        lin = np.linspace(-1.5, 1.5, g)
        for j, kk in enumerate(keep_modes):
            self.offsets[kk] = [lin[j % g], lin[j // g]]
        self.advten_in = np.tile(self.shape_norm, (MODES, 1))
        self.advten_in[:, 0] -= self.offsets[:, 0] * sx
        self.advten_in[:, 2] -= self.offsets[:, 1] * sy
        # bases of the advection network's second channel, [kept modes][2N]
        th = torch.arange(N, dtype=torch.float64, device=self.device) * (2 * math.pi / N)
        k = (self.modes.double() + 1)[:, None]
        self.basis = torch.cat([torch.cos(k * th), torch.sin(k * th)], 1).float() / N

    # -- batches in each network's normalised input/output ------------------------
    def _xy(self, idx, norm):
        X = self.Xs[idx].float()
        return torch.stack([(X[:, :N] - norm[0]) / norm[1], (X[:, N:] - norm[2]) / norm[3]], 1)

    def relax_batch(self, idx):
        x = self._xy(idx, self.shape_norm)
        d = self.relax[idx]
        q = self.relax_out
        t = torch.stack([(d[:, :N] - q[0]) / q[1], (d[:, N:] - q[2]) / q[3]], 1)
        return x, t

    def selften_batch(self, idx):
        x = self._xy(idx, self.shape_norm)
        q = self.selften_out
        return x, ((self.selften[idx] - q[0]) / q[1])[:, None]

    def adv_batch(self, idx, mj):
        """idx: shape indices, mj: positions in the kept-mode list."""
        X = self.Xs[idx].float()
        q = self.shape_norm
        coords = torch.cat([(X[:, :N] - q[0]) / q[1], (X[:, N:] - q[2]) / q[3]], 1)
        x = torch.stack([coords, self.basis[mj]], 1)
        kk = self.modes[mj]
        o = torch.as_tensor(self.adv_out, dtype=torch.float32, device=self.device)[kk]
        y = self.adv[idx, mj]
        t = torch.stack([(y[:, 0] - o[:, 0:1]) / o[:, 1:2], (y[:, 1] - o[:, 2:3]) / o[:, 3:4]], 1)
        return x, t

    def advten_batch(self, idx, mj):
        X = self.Xs[idx].float()
        kk = self.modes[mj]
        p = torch.as_tensor(self.advten_in, dtype=torch.float32, device=self.device)[kk]
        x = torch.stack([(X[:, :N] - p[:, 0:1]) / p[:, 1:2], (X[:, N:] - p[:, 2:3]) / p[:, 3:4]], 1)
        o = torch.as_tensor(self.advten_out, dtype=torch.float32, device=self.device)[kk]
        y = self.advten[idx, mj]
        t = torch.stack([(y[:, 0] - o[:, 0:1]) / o[:, 1:2], (y[:, 1] - o[:, 2:3]) / o[:, 3:4]], 1)
        return x, t

    def norms(self):
        """The ten arrays of the reference constructor (MLARM_manyfree_py)."""
        return {"adv_in": self.adv_in, "adv_out": self.adv_out, "relax_in": self.shape_norm.copy(),
                "relax_out": self.relax_out, "selften_in": self.shape_norm.copy(), "selften_out": self.selften_out,
                "advten_in": self.advten_in, "advten_out": self.advten_out}


# ---------------------------------------------------------------------------
# training loops

def _lr(step, total, lr0, warm=200):
    if step < warm:
        return lr0 * (step + 1) / warm
    return lr0 * 0.5 * (1.0 + math.cos(math.pi * min(1.0, (step - warm) / max(1, total - warm))))


def train_network(name: str, data: Dataset, train_idx: torch.Tensor, seconds: float, batch: int = 256,
                  lr: float = 5e-4, seed: int = 0, log=None):
    """Train the one-group network ``name`` for about ``seconds`` of wall
    clock (cosine schedule over the steps the first ones' rate allows)."""
    spec = group_spec(name)
    if train_idx.numel() == 0 or int(train_idx.min()) < 0 or int(train_idx.max()) >= data.n:
        raise IndexError(f"train_network: sample indices outside the {data.n} shapes of the dataset")
    tr = Trainer(spec, init_state_dict(spec, seed), "fp32", batch, data.device)
    gen = torch.Generator(data.device).manual_seed(seed + 1)
    nmodes = len(data.modes)

    def sample():
        idx = train_idx[torch.randint(0, train_idx.numel(), (batch,), device=data.device, generator=gen)]
        if name in ("relax", "selften"):
            return getattr(data, name + "_batch")(idx)
        mj = torch.randint(0, nmodes, (batch,), device=data.device, generator=gen)
        return getattr(data, name + "_batch")(idx, mj)

    def weights(t):
        # the loss as a relative error: each sample weighted by its inverse
        # mean square (floor 0.2 of the normalised scale: weights <= 5)
        return 1.0 / torch.clamp((t.double() ** 2).mean(dim=(1, 2)), min=0.2)

    # rate probe: 20 steps after 5 (the first launches load the kernels)
    for i in range(25):
        if i == 5:
            torch.cuda.synchronize(data.device)
            t0 = time.perf_counter()
        x, t = sample()
        tr.train_step(x, t, _lr(i, 10 ** 9, lr), sample_weights=weights(t))
    torch.cuda.synchronize(data.device)
    per = (time.perf_counter() - t0) / 20
    total = max(50, int(seconds / per))
    losses = []
    for i in range(25, total):
        x, t = sample()
        want = (i % 200 == 0) or i == total - 1
        loss = tr.train_step(x, t, _lr(i, total, lr), want_loss=want, sample_weights=weights(t))
        if want:
            losses.append((i, loss))
            if log:
                log(f"{name}: step {i}/{total} loss {loss:.3e}")
    return tr, {"steps": total, "s_per_step": per, "losses": losses}


def evaluate(name: str, tr: Trainer, data: Dataset, idx: torch.Tensor, batch: int = 256):
    """Relative error (2-norm over the samples) of the de-normalised network
    outputs against the BIEM targets on samples ``idx`` (all kept modes)."""
    if idx.numel() == 0 or int(idx.min()) < 0 or int(idx.max()) >= data.n:
        raise IndexError(f"evaluate: sample indices outside the {data.n} shapes of the dataset")
    num = den = 0.0
    batch = min(batch, tr.max_batch)
    for a in range(0, idx.numel(), batch):
        ib = idx[a:a + batch]
        if name in ("relax", "selften"):
            x, t = getattr(data, name + "_batch")(ib)
            y = tr.forward(x)
            q = data.relax_out if name == "relax" else data.selften_out
            if name == "relax":
                sc = torch.tensor([q[1], q[3]], dtype=torch.float32, device=data.device)[None, :, None]
                e, r = (y - t) * sc, t * sc + torch.tensor([q[0], q[2]], dtype=torch.float32,
                                                           device=data.device)[None, :, None]
            else:
                e, r = (y - t) * q[1], t * q[1] + q[0]
            num += float((e.double() ** 2).sum())
            den += float((r.double() ** 2).sum())
        else:
            for j in range(len(data.modes)):
                mj = torch.full((ib.numel(),), j, dtype=torch.long, device=data.device)
                x, t = getattr(data, name + "_batch")(ib, mj)
                y = tr.forward(x)
                o = (data.adv_out if name == "adv" else data.advten_out)[int(data.modes[j])]
                sc = torch.tensor([o[1], o[3]], dtype=torch.float32, device=data.device)[None, :, None]
                mu = torch.tensor([o[0], o[2]], dtype=torch.float32, device=data.device)[None, :, None]
                num += float((((y - t) * sc).double() ** 2).sum())
                den += float(((t * sc + mu).double() ** 2).sum())
    return math.sqrt(num / max(den, 1e-300))


def save(out_dir: str, nets: dict, norms: dict, meta: dict):
    """Write the trained one-group weights (float16, ``{name}.npz``), the
    normalisation arrays (``norms.npz``) and a summary (``train_log.json``)."""
    import json
    os.makedirs(out_dir, exist_ok=True)
    for name, sd in nets.items():
        np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), **{k: v.astype(np.float16) for k, v in sd.items()})
    np.savez(os.path.join(out_dir, "norms.npz"), **{k: np.asarray(v, dtype=np.float64) for k, v in norms.items()})
    with open(os.path.join(out_dir, "train_log.json"), "w") as f:
        json.dump(meta, f, indent=1)


def load(model_dir: str = TRAINED_DIR):
    """(state_dicts of the five merged networks, normalisation arrays) from
    ``model_dir``; networks without a trained file keep the seeded synthetic
    weights (the near-field network, whose output the step reads only
    through the repulsion force)."""
    from .mlarm_weights import synthetic_norms, synthetic_state_dict
    nz = np.load(os.path.join(model_dir, "norms.npz"))
    norms = {k: nz[k] for k in nz.files}
    syn = synthetic_norms(0)
    for k in ("near_in", "near_out"):
        norms.setdefault(k, syn[k])
    sds = {}
    for name in NETS:
        p = os.path.join(model_dir, f"{name}.npz")
        if os.path.exists(p):
            g = np.load(p)
            sds[name] = merge_groups(name, {k: g[k].astype(np.float32) for k in g.files})
        else:
            sds[name] = synthetic_state_dict(name, 0)
    return sds, norms


def have_trained(model_dir: str = TRAINED_DIR) -> bool:
    return os.path.exists(os.path.join(model_dir, "norms.npz"))


def surrogate_errors(nets: dict, norms: dict, Xs: torch.Tensor, modes=TRAIN_MODES, dt: float = 1e-5):
    """The plain BIEM operators as the judge of the surrogate: relative errors
    (2-norm over the vesicles and points) of the merged networks ``nets``
    (mlarm.Network objects, as the step runs them) against ves_mlarm_targets
    on standardised shapes Xs[nv][2N] (device).  The networks' inputs and
    outputs are normalised and de-normalised as the step does
    (get_network_torch.py pre/post-processing); the merged networks are
    compared on the Fourier modes ``modes``."""
    dev = Xs.device
    nv = Xs.shape[0]
    t = targets(Xs, dt)
    x, y = Xs[:, :N], Xs[:, N:]

    def q(name):
        return torch.as_tensor(np.asarray(norms[name], dtype=np.float64), device=dev)

    def rel(a, b):
        return float(torch.linalg.norm((a - b).reshape(-1)) / torch.linalg.norm(b.reshape(-1)))

    out = {}
    p, o = q("relax_in"), q("relax_out")
    inp = torch.stack([(x - p[0]) / p[1], (y - p[2]) / p[3]], 1)
    r = nets["relax"](inp).double()
    dx = torch.cat([r[:, 0] * o[1] + o[0], r[:, 1] * o[3] + o[2]], 1) * (dt / 1e-5)
    out["relax"] = rel(dx, t["relax"])
    p, o = q("selften_in"), q("selften_out")
    inp = torch.stack([(x - p[0]) / p[1], (y - p[2]) / p[3]], 1)
    out["selften"] = rel(nets["selften"](inp).double()[:, 0] * o[1] + o[0], t["selften"])
    km = torch.tensor(modes, dtype=torch.long, device=dev)
    # advection-tension: channel 2k + c is coordinate c normalised with mode k's statistics
    p, o = q("advten_in"), q("advten_out")
    inp = torch.stack([(x[:, None, :] - p[None, :, 0, None]) / p[None, :, 1, None],
                       (y[:, None, :] - p[None, :, 2, None]) / p[None, :, 3, None]], 2).reshape(nv, 2 * MODES, N)
    z = nets["advten"](inp).double().reshape(nv, MODES, 2, N)
    z = torch.stack([z[:, :, 0] * o[None, :, 1, None] + o[None, :, 0, None],
                     z[:, :, 1] * o[None, :, 3, None] + o[None, :, 2, None]], 2)
    out["advten"] = rel(z[:, km], t["advten"].reshape(nv, MODES, 2, N)[:, km])
    # advection: channel 2k = [x ++ y] normalised (mode 63: unit std), 2k + 1 = the mode's basis
    p, o = q("adv_in"), q("adv_out")
    sx = p[:, 1].clone()
    sy = p[:, 3].clone()
    sx[NYQUIST] = 1.0
    sy[NYQUIST] = 1.0
    coords = torch.cat([(x[:, None, :] - p[None, :, 0, None]) / sx[None, :, None],
                        (y[:, None, :] - p[None, :, 2, None]) / sy[None, :, None]], 2)
    th = torch.arange(N, dtype=torch.float64, device=dev) * (2 * math.pi / N)
    kk = torch.arange(1, MODES + 1, dtype=torch.float64, device=dev)[:, None]
    basis = torch.cat([torch.cos(kk * th), torch.sin(kk * th)], 1) / N
    inp = torch.stack([coords, basis[None].expand(nv, -1, -1)], 2).reshape(nv, 2 * MODES, 2 * N)
    w = nets["adv"](inp).double().reshape(nv, MODES, 2, 2 * N)
    w = torch.stack([w[:, :, 0] * o[None, :, 1, None] + o[None, :, 0, None],
                     w[:, :, 1] * o[None, :, 3, None] + o[None, :, 2, None]], 2)
    out["adv"] = rel(w[:, km], t["adv"].reshape(nv, MODES, 2, 2 * N)[:, km])
    return out
