"""The MLARM oracle against fixtures recorded from the reference (CPU only).

Fixtures (tests/golden/make_golden.py): ``nets_fp64`` holds each network's
output on seeded inputs from the reference model classes in FP64;
``mlarm_fp64`` two reference MLARM steps with everything in FP64 plus the
stage outputs of the first; ``mlarm_mixed`` the same run with FP64 geometry
and the reference's FP32 networks.  Network weights and normalisation
constants are the seeded synthetic ones of ``ves2dpy_gb300.mlarm_weights``.
"""
import functools

import numpy as np
import pytest

from oracle import mlarm_oracle as M
from ves2dpy_gb300.mlarm_weights import NETS, net_test_input, synthetic_norms, synthetic_state_dict


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@functools.lru_cache(maxsize=1)
def _nets():
    return M.Nets({n: synthetic_state_dict(n, 0) for n in NETS}, synthetic_norms(0))


def test_eig2_matches_lapack_convention():
    import torch
    rng = np.random.default_rng(0)
    for _ in range(2000):
        a, b, d = rng.normal(size=3) * rng.choice([1e-3, 1.0, 1e3], size=3)
        w, V = M.eig2_lapack(a, b, b, d)
        wt, Vt = torch.linalg.eig(torch.tensor([[a, b], [b, d]], dtype=torch.float64))
        np.testing.assert_allclose(w, wt.real.numpy(), rtol=1e-12, atol=1e-12 * max(abs(a), abs(b), abs(d)))
        np.testing.assert_allclose(V, Vt.real.numpy(), rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", list(NETS))
def test_network_forward_matches_reference_modules(golden, name):
    g = golden("nets_fp64")
    spec = NETS[name]
    y = M.net_forward(spec, synthetic_state_dict(name, 0), net_test_input(name))
    co = spec.cout
    ys = np.stack([y[:, k * co:(k + 1) * co] for k in g[name + "_groups"]], axis=1)
    assert rel(ys, g[name]) < 1e-12


def test_standardization_matches_reference(golden):
    g = golden("mlarm_fp64")
    Xs, sv = M.standardization_step(g["Xinit"])
    assert rel(Xs, g["stand_X"]) < 1e-12
    for k, v in zip(("scaling", "rotate", "rotCenter", "trans"), sv):
        assert rel(v, g["stand_" + k]) < 1e-12, k
    assert np.array_equal(sv[4], g["stand_sortIdx"])


def test_mlarm_step_stages_and_two_steps_match_reference(golden):
    g = golden("mlarm_fp64")
    nets = _nets()
    rec = {}
    X1, t1 = M.mlarm_step(nets, g["Xinit"], np.zeros((128, 4)), g["area0"], g["len0"], record=rec)
    for i in range(3):
        assert np.array_equal(np.asarray(rec["excl"][i]), g[f"near_ids{i}"])
    for k in ("far1", "far2", "vback_solve", "selfbend_solve", "Xadv", "Xrelax", "Xalign", "Xcorr"):
        assert rel(rec[k], g[k]) < 1e-11, k
    assert rel(X1, g["X1"]) < 1e-12
    assert rel(t1, g["ten1"]) < 1e-11
    X2, t2 = M.mlarm_step(nets, X1, t1, g["area0"], g["len0"])
    assert rel(X2, g["X2"]) < 1e-12
    assert rel(t2, g["ten2"]) < 1e-11


def test_mlarm_step_close_to_reference_with_fp32_networks(golden):
    """The reference as its driver configures it (FP32 networks): the FP64
    oracle stays within FP32 network noise of it."""
    g = golden("mlarm_mixed")
    X1, t1 = M.mlarm_step(_nets(), g["Xinit"], np.zeros((128, 4)), g["area0"], g["len0"])
    assert rel(X1, g["X1"]) < 1e-4
    assert rel(t1, g["ten1"]) < 1e-3
