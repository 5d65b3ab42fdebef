"""GPU parity of the MLARM path: the network engine and the whole step.

References: ``tests/golden/nets_fp64.npz`` (reference model classes, FP64),
``mlarm_fp64.npz`` (two reference MLARM steps, everything FP64) and
``mlarm_mixed.npz`` (FP64 geometry, the reference's FP32 networks).
Weights and normalisation constants are the seeded synthetic ones.
"""
import functools

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@functools.lru_cache(maxsize=1)
def _state_dicts():
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_state_dict
    return {n: synthetic_state_dict(n, 0) for n in NETS}


@functools.lru_cache(maxsize=3)
def _mlarm(net_precision, farfield_precision):
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.mlarm import MLARM_manyfree_py
    from ves2dpy_gb300.mlarm_weights import synthetic_norms
    nrm = {k: torch.from_numpy(v) for k, v in synthetic_norms(0).items()}

    def vinf(X):
        N = X.shape[0] // 2
        return 2.0 * torch.vstack((X[N:], torch.zeros_like(X[:N])))

    return MLARM_manyfree_py(1e-5, vinf, Curve(), False, 1e2, -1,
                             nrm["adv_in"], nrm["adv_out"], nrm["relax_in"], nrm["relax_out"],
                             nrm["near_in"], nrm["near_out"], nrm["selften_in"], nrm["selften_out"],
                             nrm["advten_in"], nrm["advten_out"], DEV, state_dicts=_state_dicts(),
                             net_precision=net_precision, farfield_precision=farfield_precision)


# FP64 engine: summation order only; FP32 engine: the reference networks' own
# type; BF16 tensor-core engine: BF16 operands (8-bit mantissa) with FP32
# accumulation and FP32 activations between blocks, relative to the largest
# output of the network (the self-tension network's single output channel is
# the least well conditioned)
NET_TOL = {"fp64": 1e-12, "fp32": 1e-4, "bf16": 3e-2}


@pytest.mark.parametrize("precision", ["fp64", "fp32", "bf16"])
@pytest.mark.parametrize("name", ["relax", "adv", "near", "selften", "advten"])
def test_network_engine_matches_reference(golden, name, precision):
    from ves2dpy_gb300.mlarm import Network
    from ves2dpy_gb300.mlarm_weights import NETS, net_test_input
    g = golden("nets_fp64")
    spec = NETS[name]
    net = Network(name, _state_dicts()[name], precision, DEV)
    y = net(torch.from_numpy(net_test_input(name))).double().cpu().numpy()
    co = spec.cout
    ys = np.stack([y[:, k * co:(k + 1) * co] for k in g[name + "_groups"]], axis=1)
    err = rel(ys, g[name])
    assert err < NET_TOL[precision], (name, precision, err)


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_network_engine_batch_of_vesicles(precision):
    """Vesicles are independent: a batch equals its members run alone, bit for bit."""
    from ves2dpy_gb300.mlarm import Network
    from ves2dpy_gb300.mlarm_weights import net_test_input
    net = Network("advten", _state_dicts()["advten"], precision, DEV)
    x = torch.from_numpy(net_test_input("advten", nv=3, seed=11))
    yb = net(x)
    for v in range(3):
        assert torch.equal(net(x[v:v + 1]), yb[v:v + 1])


def test_standardization_matches_reference(golden):
    g = golden("mlarm_fp64")
    m = _mlarm("fp64", "fp64")
    Xs, (sc, rot, rc, tr, si) = m.standardizationStep(torch.from_numpy(g["Xinit"]).to(DEV))
    assert rel(Xs, g["stand_X"]) < 1e-10
    assert rel(sc, g["stand_scaling"]) < 1e-12
    assert rel(rot, g["stand_rotate"]) < 1e-10
    assert rel(rc, g["stand_rotCenter"]) < 1e-10
    assert rel(tr, g["stand_trans"]) < 1e-10
    assert np.array_equal(si.cpu().numpy(), g["stand_sortIdx"])


def test_mlarm_step_fp64_matches_reference(golden):
    """FP64 networks and far field: every stage of the first step and each of
    the recorded steps (10) at 1e-10."""
    g = golden("mlarm_fp64")
    m = _mlarm("fp64", "fp64")
    m.area0 = torch.from_numpy(g["area0"])
    m.len0 = torch.from_numpy(g["len0"])
    X0 = torch.from_numpy(g["Xinit"]).to(DEV)
    t = m.time_step_trace(X0, torch.zeros(128, 4, dtype=torch.float64, device=DEV))
    assert m.last_result.n_near_pairs == len(g["near_ids0"])
    for k in ("far1", "far2", "vback_solve", "selfbend_solve", "Xadv", "Xrelax", "Xalign", "Xcorr"):
        assert rel(t[k], g[k]) < 1e-10, (k, rel(t[k], g[k]))
    assert rel(t["X"], g["X1"]) < 1e-10
    assert rel(t["ten"], g["ten1"]) < 1e-10
    X, ten = t["X"], t["ten"]
    nsteps = int(g["nsteps"]) if "nsteps" in g.files else 2
    for step in range(2, nsteps + 1):
        X, ten = m.time_step_many_noinfo(X, ten, 3)
        assert rel(X, g[f"X{step}"]) < 1e-10, (step, rel(X, g[f"X{step}"]))
        assert rel(ten, g[f"ten{step}"]) < 1e-10, (step, rel(ten, g[f"ten{step}"]))


def test_autotuned_launch_shapes_give_the_fixed_rule_outputs():
    """The autotuner (ves_net_set_autotune) only picks among launch shapes of
    the same arithmetic: its outputs equal the fixed rule's bit for bit, on
    the timing pass and after it."""
    from ves2dpy_gb300.mlarm import Network
    from ves2dpy_gb300.mlarm_weights import net_test_input
    for name in ("adv", "near"):
        sd = _state_dicts()[name]
        x = torch.from_numpy(net_test_input(name, nv=48, seed=21))
        y0 = Network(name, sd, "bf16", DEV, autotune=False)(x)
        tuned = Network(name, sd, "bf16", DEV, autotune=True)
        y1 = tuned(x)
        y2 = tuned(x)
        assert torch.equal(y0, y1), name
        assert torch.equal(y0, y2), name


def test_mlarm_step_fp32_networks(golden):
    """FP32 networks and the compensated FP32 far field, against the FP64
    reference and against the reference with its own FP32 networks."""
    m = _mlarm("fp32", "fp32c")
    for fixture, tol_x, tol_t in (("mlarm_fp64", 1e-4, 1e-3), ("mlarm_mixed", 1e-4, 1e-3)):
        g = golden(fixture)
        m.area0 = torch.from_numpy(g["area0"])
        m.len0 = torch.from_numpy(g["len0"])
        X1, t1 = m.time_step_many_noinfo(torch.from_numpy(g["Xinit"]).to(DEV),
                                         torch.zeros(128, 4, dtype=torch.float64, device=DEV), 3)
        assert rel(X1, g["X1"]) < tol_x, (fixture, rel(X1, g["X1"]))
        assert rel(t1, g["ten1"]) < tol_t, (fixture, rel(t1, g["ten1"]))


@pytest.mark.parametrize("farfield", ["fp32c", "fp32m"])
def test_mlarm_step_bf16_networks(golden, farfield):
    """Tensor-core networks: the step stays within BF16 network noise of the
    FP64 reference (the networks move the shape by dt * velocity and the
    relaxation by a 2e-4-scaled correction, so the shape error is small while
    the predicted tension carries the networks' relative error).  Both FP32
    all-pairs paths (direct, multipole) keep the far field within 1e-5."""
    g = golden("mlarm_fp64")
    m = _mlarm("bf16", farfield)
    m.area0 = torch.from_numpy(g["area0"])
    m.len0 = torch.from_numpy(g["len0"])
    t = m.time_step_trace(torch.from_numpy(g["Xinit"]).to(DEV), torch.zeros(128, 4, dtype=torch.float64, device=DEV))
    assert rel(t["far1"], g["far1"]) < 1e-5          # geometry only: FP32 far field
    assert rel(t["X"], g["X1"]) < 1e-4, rel(t["X"], g["X1"])
    assert rel(t["ten"], g["ten1"]) < 5e-2, rel(t["ten"], g["ten1"])


def test_biem_fallback_is_the_biem_step_of_the_vesicle():
    """judge_tol: with a tolerance nothing meets, a vesicle takes the implicit
    BIEM step of the isolated vesicle with the step's explicit velocity.  A
    single vesicle has no far field, so that velocity is the background flow
    and the fallback shape (the step's relaxed shape before the
    re-parametrisation and conditioning) is the plain BIEM step's result,
    whatever the networks predict; with a tolerance everything meets, the
    step is the surrogate's, bit for bit."""
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.training import random_shapes
    from ves2dpy_gb300.tstep_biem import TStepBiem
    x = random_shapes(1, 21, reduced_area=(0.65, 0.65), amp=(0.02, 0.02))[0]
    X = torch.from_numpy(np.concatenate([x[:128], x[128:] + 3.0])[:, None].copy()).to(DEV)
    ten = torch.zeros(128, 1, dtype=torch.float64, device=DEV)
    m = _mlarm("bf16", "fp32m")
    _, a0, l0 = Curve().geomProp(X)
    m.area0, m.len0 = a0, l0
    try:
        m.judge_tol = 0.0
        Xs, _ = m.time_step_many_noinfo(X, ten, 3)
        m.judge_tol = 1e10
        Xj, _ = m.time_step_many_noinfo(X, ten, 3)
        assert m.last_result.n_fallback == 0
        assert torch.equal(Xs, Xj)
        m.judge_tol = 1e-300
        tr = m.time_step_trace(X, ten)
        assert m.last_result.n_fallback == 1
    finally:
        m.judge_tol = 0.0
    prams = dict(dt=1e-5, kappa=1.0, gmresTol=1e-13, gmresMaxIter=100, farFieldSpeed=2.0, viscCont=[1.0])
    tt = TStepBiem(X, None, dict(farField="shear", usePreco=True), prams, near="py_hh", farfield_precision="fp32m",
                   sl_precision="fp32c")
    Xb, *_ = tt.time_step(X, ten)
    assert rel(tr["Xrelax"], Xb.cpu()) < 1e-10


def test_conserve_keeps_area_and_length():
    """conserve: the advection displacement loses its first-order area and
    length changes.  In shear flow the seeded networks' inextensibility
    correction is tiny, so the advected shape stretches at first order in dt;
    with conserve on, only the second-order change is left."""
    import math
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.suspension import random_suspension
    X0 = random_suspension(16, 128, 0.05, min_gap=0.1, area=0.65 / (4 * math.pi), seed=6)
    X = torch.from_numpy(X0).to(DEV)
    ten = torch.zeros(128, 16, dtype=torch.float64, device=DEV)
    m = _mlarm("bf16", "fp32m")
    cv = Curve()
    _, a0, l0 = cv.geomProp(X)
    m.area0, m.len0 = a0, l0
    change = {}
    try:
        for flag in (False, True):
            m.conserve = flag
            Xadv = m.time_step_trace(X, ten)["Xadv"]
            _, a, l = cv.geomProp(Xadv)
            change[flag] = max(float(((a - a0) / a0).abs().max()), float(((l - l0) / l0).abs().max()))
    finally:
        m.conserve = False
    assert change[True] < 0.05 * change[False], change
