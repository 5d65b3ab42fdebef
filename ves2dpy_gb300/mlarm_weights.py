"""Network specifications and weights for the five MLARM networks.

The reference loads trained TorchScript models from
``../trained/torch_script_models/*.pt`` (``newtorch/wrapper_MLARM_batch_compile_N128.py:671-707``);
the files are not part of the reference tree.  This module describes the
five architectures in the terms the device engine needs, reads a state dict
in the reference's parameter naming (``model.state_dict()`` of the
TorchScript module), and generates seeded synthetic weights and
normalisation constants with the same names and shapes for benchmarks and
parity tests.

Every network is a chain of identical block templates
(``model_zoo/Net_ves_merge_adv.py:6-191`` and siblings), applied to ``rep``
independent channel groups (grouped convolutions, ``groups=rep``):

    a = relu(conv7_s2(x)) ++ relu(conv7_s2_dil2(x))   ->  bn1   (2*c1 channels, L/2)
    b = relu(conv7_s2(a)) ++ relu(conv7_s2_dil2(a))   ->  bn2   (2*c2 channels, L/4)
    c = bn3(relu(deconv10_s2(b)))                             (2*c2, L/2)
    d = bn4(relu(deconv10_s2(c)))                             (2*c2, L)
    m = mix3(d)                                               (cmix, L)
    out = [m + x[:cmix] if residual else m] ++ x[cin-npass:cin]

The synthetic generator is a counter-based SplitMix64 stream keyed by
(seed, parameter name), so that the same weights are produced bit-for-bit on
any machine without storing them.
"""
from __future__ import annotations

import math
import zlib
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class BlockSpec:
    prefix: str      # state-dict prefix, e.g. "layers.3" or "starter"
    cin: int         # input channels per group
    c1: int          # output channels of each first-stage convolution
    c2: int          # output channels of each second-stage convolution
    cmix: int        # output channels of the mixing convolution
    residual: bool   # out[:cmix] += x[:cmix]
    npass: int       # input channels appended unchanged after the mix output

    @property
    def cout(self) -> int:
        return self.cmix + self.npass


@dataclass(frozen=True)
class NetSpec:
    name: str
    rep: int         # channel groups (Fourier modes for the merged networks)
    L: int           # signal length
    blocks: tuple    # BlockSpec, in execution order

    @property
    def cin(self) -> int:
        return self.blocks[0].cin

    @property
    def cout(self) -> int:
        return self.blocks[-1].cout


def _f(x):
    return int(math.floor(x))


def _chain(layer_prefix, nblocks, factor, ch, start_pass, evo_res_pass, end_out, start_cin=2):
    """Starter + (nblocks-1) Evo + End, the layout of the merged/self-tension nets."""
    c2 = _f(10 * factor)
    blocks = [BlockSpec("starter", start_cin, _f(9 * factor), c2, ch, False, start_pass)]
    ecin = ch + start_pass
    for i in range(nblocks - 1):
        blocks.append(BlockSpec(f"{layer_prefix}.{i}", ecin, _f(8 * factor), c2, ch, True, evo_res_pass))
    blocks.append(BlockSpec("end", ecin, _f(8 * factor), c2, end_out, False, 0))
    return tuple(blocks)


def _relax_blocks(nblocks, factor):
    """pdeNet_Ves_factor_periodic (model_zoo/Net_ves_factor.py:6-56): Evo blocks, x + mix."""
    return tuple(BlockSpec(f"layer.{i}", 2, _f(8 * factor), _f(10 * factor), 2, True, 0) for i in range(nblocks))


# Architectures as instantiated by model_zoo/get_network_torch.py
NETS = {
    # RelaxNetwork: pdeNet_Ves_factor_periodic(14, 2.9)  (get_network_torch.py:28)
    "relax": NetSpec("relax", 1, 128, _relax_blocks(14, 2.9)),
    # MergedAdvNetwork: Net_merge_advection(12, 1.7, 20, rep=127)  (:137); Net_ves_merge_adv.py
    "adv": NetSpec("adv", 127, 256, _chain("layers", 12, 1.7, 20, 1, 1, 2)),
    # TenSelfNetwork: Net_ves_selften(12, 2.4, 26)  (:217); Net_ves_selften.py
    "selften": NetSpec("selften", 1, 128, _chain("layer", 12, 2.4, 26, 2, 2, 1)),
    # MergedTenAdvNetwork: Net_ves_merge_advten(12, 2.5, 24, rep=127)  (:316); Net_ves_merge_advten.py
    "advten": NetSpec("advten", 127, 128, _chain("layer", 12, 2.5, 24, 0, 0, 2)),
    # MergedNearFourierNetwork ("disth" model): Net_ves_merge_nocoords_nearFourier(13, 3.0, 26, rep=128) (:404)
    "near": NetSpec("near", 128, 128, _chain("layer", 13, 3.0, 26, 0, 0, 12)),
}

# Reference constructor arguments, for building the reference modules in tests.
NET_ARGS = {
    "relax": (14, 2.9),
    "adv": (12, 1.7, 20, 127),
    "selften": (12, 2.4, 26),
    "advten": (12, 2.5, 24, 127),
    "near": (13, 3.0, 26, 128),
}

# File names the reference constructor loads (wrapper_MLARM_batch_compile_N128.py:671-707).
MODEL_FILES = {
    "adv": "2024Oct_ves_merged_adv.pt",
    "relax": "ves_relax_DIFF_June8_625k_dt1e-5.pt",
    "near": "ves_merged_disth_nearFourier.pt",
    "selften": "Ves_2024Oct_selften_12blks_loss_0.00566cuda1.pt",
    "advten": "2024Oct_ves_merged_advten.pt",
}

_CONVS = ("conv1_1", "conv1_2", "conv2_1", "conv2_2", "deconv1", "deconv2", "mix")
_BNS = ("bn1", "bn2", "bn3", "bn4")


def param_shapes(spec: NetSpec):
    """(name, shape, fan_in) of every parameter and buffer the engine reads."""
    G = spec.rep
    out = []
    for b in spec.blocks:
        d = 2 * b.c2
        conv = {
            "conv1_1": ((b.c1 * G, b.cin, 7), b.cin * 7),
            "conv1_2": ((b.c1 * G, b.cin, 7), b.cin * 7),
            "conv2_1": ((b.c2 * G, 2 * b.c1, 7), 2 * b.c1 * 7),
            "conv2_2": ((b.c2 * G, 2 * b.c1, 7), 2 * b.c1 * 7),
            "deconv1": ((d * G, d, 10), d * 10),
            "deconv2": ((d * G, d, 10), d * 10),
            "mix": ((b.cmix * G, d, 3), d * 3),
        }
        bnf = {"bn1": 2 * b.c1 * G, "bn2": d * G, "bn3": d * G, "bn4": d * G}
        for name in _CONVS:
            shp, fan = conv[name]
            nout = shp[0] if name not in ("deconv1", "deconv2") else shp[1] * G
            out.append((f"{b.prefix}.{name}.weight", shp, fan))
            out.append((f"{b.prefix}.{name}.bias", (nout,), fan))
        for name in _BNS:
            for field in ("weight", "bias", "running_mean", "running_var"):
                out.append((f"{b.prefix}.{name}.{field}", (bnf[name],), 0))
    return out


def _splitmix_uniform(seed: int, key: str, n: int) -> np.ndarray:
    """n uniforms in [0, 1) from SplitMix64 at counters 0..n-1 of stream (seed, key)."""
    base = (np.uint64(seed & 0xFFFFFFFF) << np.uint64(32)) ^ np.uint64(zlib.crc32(key.encode()))
    with np.errstate(over="ignore"):
        z = base * np.uint64(0x9E3779B97F4A7C15) + (np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def synthetic_state_dict(net: str, seed: int = 0):
    """Seeded weights in the reference naming and shapes (float32 arrays).

    Convolutions follow the uniform(+-1/sqrt(fan_in)) scale of PyTorch's
    default initialisation; batch-norm affine parameters and running
    statistics are drawn around (1, 0, 0, 1) so that every term of the
    eval-mode normalisation is exercised.
    """
    spec = NETS[net]
    sd = {}
    for name, shape, fan in param_shapes(spec):
        n = int(np.prod(shape))
        u = _splitmix_uniform(seed, f"{net}/{name}", n)
        if name.endswith("running_var"):
            v = 0.5 + u
        elif fan == 0 and name.endswith(".weight"):
            v = 0.8 + 0.4 * u
        elif fan == 0:
            v = 0.2 * (u - 0.5)
        else:
            v = (2.0 * u - 1.0) / math.sqrt(fan)
        sd[name] = v.reshape(shape).astype(np.float32)
    return sd


def synthetic_norms(seed: int = 0):
    """Normalisation constants with the shapes the reference constructor takes
    (entry_driver_manyfreeSpaceVesicle_N128.py:120-145), float64.

    Input statistics are those of unit-length shapes (mean ~0, std ~0.06 in x
    and ~0.13 in y); output scales keep every surrogate term of one step small
    compared with the shape, as the trained networks do.
    """
    def u(key, shape):
        return _splitmix_uniform(seed, "norm/" + key, int(np.prod(shape))).reshape(shape)

    def stats(key, modes, std_lo, std_hi):
        r = u(key, (modes, 4))
        out = np.empty((modes, 4))
        out[:, 0] = 1e-3 * (r[:, 0] - 0.5)
        out[:, 1] = std_lo[0] + (std_hi[0] - std_lo[0]) * r[:, 1]
        out[:, 2] = 1e-3 * (r[:, 2] - 0.5)
        out[:, 3] = std_lo[1] + (std_hi[1] - std_lo[1]) * r[:, 3]
        return out

    nin = stats("near_in", 128, (0.05, 0.1), (0.07, 0.15))
    r = u("near_out", (128, 2, 12))
    nout = np.empty((128, 2, 12))
    nout[:, 0] = 1e-4 * (r[:, 0] - 0.5)
    nout[:, 1] = 1e-4 * (0.5 + r[:, 1])
    return {
        "adv_in": stats("adv_in", 127, (0.05, 0.1), (0.07, 0.15)),
        "adv_out": stats("adv_out", 127, (2e-6, 2e-6), (6e-6, 6e-6)),
        "relax_in": np.array([0.0, 0.0628, 0.0, 0.1334]),
        "relax_out": np.array([0.0, 2.0e-4, 0.0, 1.8e-4]),
        "near_in": nin,
        "near_out": nout,
        "selften_in": np.array([2e-4, 0.0628, 2e-3, 0.1334]),
        "selften_out": np.array([340.0, 470.0]),
        "advten_in": stats("advten_in", 127, (0.05, 0.1), (0.07, 0.15)),
        "advten_out": stats("advten_out", 127, (1e-3, 1e-3), (3e-3, 3e-3)),
    }


def net_test_input(net: str, nv: int = 1, seed: int = 7) -> np.ndarray:
    """Seeded float64 input (nv, rep*cin, L) in [-1, 1) for network parity tests."""
    spec = NETS[net]
    shape = (nv, spec.rep * spec.cin, spec.L)
    return (2.0 * _splitmix_uniform(seed, "input/" + net, int(np.prod(shape))) - 1.0).reshape(shape)
