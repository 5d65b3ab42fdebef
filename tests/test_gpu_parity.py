"""GPU parity of the C-ABI kernels against the reference golden fixtures and
the FP64 oracle.

Tolerances (relative, max-norm): FP64 paths 1e-10; FP32-compensated far field
1e-5; the mixed-precision Alpert matrix 1e-5.
"""
import numpy as np
import pytest
import torch

from oracle import ves2d_oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-5


def dev():
    return torch.device("cuda:0")


def T(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device=dev())


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("N", [16, 32])
def test_capsule_operators(golden, N):
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.curve import Curve
    g = golden("capsules_fp64")
    X, sig, f = g[f"X{N}"], g[f"sig{N}"], g[f"f{N}"]
    ves = capsules(T(X), None, None, 1.0, 1.0)
    assert rel(ves.sa, g[f"sa{N}"]) < FP64_TOL
    assert rel(ves.xt, g[f"xt{N}"]) < FP64_TOL
    assert rel(ves.cur, g[f"cur{N}"]) < FP64_TOL
    assert rel(ves.tracJump(T(X), T(sig)), g[f"trac{N}"]) < FP64_TOL
    assert rel(ves.surfaceDiv(T(f)), g[f"sdiv{N}"]) < FP64_TOL
    Ben, Ten, Div = ves.computeDerivs()
    assert rel(Ben, g[f"Ben{N}"]) < FP64_TOL
    assert rel(Ten, g[f"Ten{N}"]) < FP64_TOL
    assert rel(Div, g[f"Div{N}"]) < FP64_TOL
    ra, area, length = Curve().geomProp(T(X))
    assert rel(area, g[f"area{N}"]) < FP64_TOL and rel(length, g[f"len{N}"]) < FP64_TOL


@pytest.mark.parametrize("N", [16, 32])
def test_upsample(golden, N):
    from ves2dpy_gb300.filter import interpft_vec
    g = golden("capsules_fp64")
    tab = O.PotenTables(N)
    assert rel(interpft_vec(T(g[f"X{N}"]), tab.Nup), g[f"up{N}"]) < FP64_TOL


@pytest.mark.parametrize("N", [16, 32])
def test_alpert_matrix(golden, N):
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    g = golden("capsules_fp64")
    ves = capsules(T(g[f"X{N}"]), None, None, 1.0, 1.0)
    op = Poten(N)
    assert rel(op.stokesSLmatrix(ves, "fp64"), g[f"G{N}"]) < FP64_TOL
    assert rel(op.stokesSLmatrix(ves, "fp32c"), g[f"G{N}"]) < FP32_TOL


def test_near_zone_ids(golden):
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    g = golden("far_fp64")
    near = naiveNearZoneInfo(T(g["X"]), T(g["Xup"]))
    ids = near[4]
    for got, key in zip(ids, ["ids0", "ids1", "ids2"]):
        np.testing.assert_array_equal(got, g[key])
    id1, id2 = near[2]
    np.testing.assert_array_equal(id1, g["id1"])
    np.testing.assert_array_equal(id2, g["id2"])
    h1, h2 = near[3]
    np.testing.assert_array_equal(h1, g["id1_hh"])
    np.testing.assert_array_equal(h2, g["id2_hh"])


@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("fp32c", FP32_TOL)])
def test_far_field_compare(golden, prec, tol):
    from ves2dpy_gb300 import biem_support as B
    g = golden("far_fp64")
    far2 = B.allExactStokesSLTarget_compare2(T(g["Xup"]), T(g["sa_up"]), T(g["fup"]), T(g["X"]), g["ids0"],
                                             g["ids1"], g["ids2"], precision=prec)
    assert rel(far2, g["far2"]) < tol
    far0 = B.allExactStokesSLTarget_compare2(T(g["Xup"]), T(g["sa_up"]), T(g["fup"]), T(g["X"]), [], [], [],
                                             precision=prec)
    assert rel(far0, g["far_noexcl"]) < tol
    far1, ids = B.allExactStokesSLTarget_compare1(T(g["Xup"]), T(g["sa_up"]), T(g["fup"]), T(g["X"]),
                                                  precision=prec)
    assert rel(far1, g["far1"]) < tol
    for got, key in zip(ids, ["c1_ids0", "c1_ids1", "c1_ids2"]):
        np.testing.assert_array_equal(got, g[key])


def test_exact_stokes_sl_column(golden):
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    g = golden("far_fp64")
    X = T(g["X"])
    ves = capsules(X, None, None, 1.0, 1.0)
    nv = X.shape[1]
    sl = Poten(X.shape[0] // 2).exactStokesSL(ves, T(g["f"]), X[:, :1], list(range(1, nv)))
    assert rel(sl, g["exact_sl_col0"]) < FP64_TOL
    with pytest.raises(TypeError):
        Poten(X.shape[0] // 2).exactStokesSL(ves, T(g["f"]), X[:, :2], [1])


def test_near_sing_int_hh(golden):
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    g = golden("step_near_fp64")
    X = T(g["X0"])
    N = X.shape[0] // 2
    ves = capsules(X, None, None, 1.0, 1.0)
    op = Poten(N)
    G = op.stokesSLmatrix(ves, "fp64")
    near = naiveNearZoneInfo(X)
    LP, nearF = op.nearSingInt_hh(ves, T(g["f_near"]), lambda F: op.exactStokesSLdiag(ves, G, F), near, None, ves,
                                  True)
    assert rel(nearF, g["nearField"]) < FP64_TOL
    assert rel(LP, g["LP_near"]) < FP64_TOL


def _step(X, dt, speed, near="py_hh", ff="fp64", sl="fp64", sig=None):
    from ves2dpy_gb300.tstep_biem import TStepBiem
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=dt, kappa=1.0, gmresTol=1e-10, gmresMaxIter=200, farFieldSpeed=speed, viscCont=[1.0] * nv)
    options = dict(farField="shear", usePreco=True, repulsion=False)
    tt = TStepBiem(T(X), None, options, prams, near=near, farfield_precision=ff, sl_precision=sl)
    sig = torch.zeros(N, nv, dtype=torch.float64, device=dev()) if sig is None else T(sig)
    return tt.time_step(T(X), sig)


def test_time_step_config1_fp64(golden):
    """The configuration's 10 steps, each against the reference's."""
    g = golden("step_c1_fp64")
    X, sig = g["X0"], None
    nsteps = sum(1 for k in g.files if k.startswith("iter"))
    assert nsteps == 10
    for s in range(1, nsteps + 1):
        Xn, sn, _, _, it, iflag = _step(X, float(g["dt"]), float(g["speed"]), sig=sig)
        assert not iflag
        assert it == int(g[f"iter{s}"])
        assert rel(Xn, g[f"X{s}"]) < FP64_TOL
        assert rel(sn, g[f"sig{s}"]) < 1e-8
        X, sig = Xn.cpu().numpy(), sn.cpu().numpy()


def test_time_step_near_fp64(golden):
    g = golden("step_near_fp64")
    Xn, sn, _, _, it, iflag = _step(g["X0"], float(g["dt"]), float(g["speed"]))
    assert not iflag and it == int(g["iter1"])
    assert rel(Xn, g["X1"]) < FP64_TOL
    assert rel(sn, g["sig1"]) < 1e-8


def test_time_step_config1_mixed(golden):
    """FP32C far field and Alpert matrix against the FP64 reference step."""
    g = golden("step_c1_fp64")
    Xn, sn, _, _, it, iflag = _step(g["X0"], float(g["dt"]), float(g["speed"]), ff="fp32c", sl="fp32c")
    assert rel(Xn, g["X1"]) < FP32_TOL


def test_time_step_matlab_near_vs_oracle():
    """MATLAB near-singular scheme against its CPU FP64 restatement."""
    import sys
    sys.path.insert(0, "tests/golden")
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(1)
    N, nv = 16, 4
    X = np.zeros((2 * N, nv))
    for k in range(nv):
        x, y = vesicle_shape(N, rng, 0.8, area=0.06)
        X[:N, k] = x + (k % 3) * 0.32
        X[N:, k] = y + (k // 3) * 0.30
    prm = O.StepParams(dt=1e-4, speed=2.0, near="matlab")
    ref = O.time_step(X, np.zeros((N, nv)), prm, O.PotenTables(N))
    Xn, sn, _, _, it, iflag = _step(X, 1e-4, 2.0, near="matlab")
    assert not iflag
    assert abs(it - ref.iters) <= 1
    assert rel(Xn, ref.X) < 1e-9


@pytest.mark.parametrize("tag", ["unit", "big"])
def test_post_step_conditioning(golden, tag):
    from ves2dpy_gb300.curve import Curve
    g = golden("post_fp64")
    X = g[f"X_{tag}"]
    N = X.shape[0] // 2
    oc = Curve()
    assert rel(oc.getPhysicalCenter(T(X)), g[f"center_{tag}"]) < FP64_TOL
    assert np.max(np.abs(oc.getIncAngle(T(X)).cpu().numpy() - g[f"incangle_{tag}"])) < FP64_TOL
    modes = torch.cat((torch.arange(0, N // 2), torch.arange(-N // 2, 0)))
    X1, good = oc.redistributeArcLength(T(X), modes)
    assert not good
    X5 = T(X)
    for _ in range(5):
        X5, _ = oc.redistributeArcLength(X5, modes)
    # unit-length curves are what the reference's 2*pi slope assumes; on longer
    # curves each pass amplifies round-off (1e-16 -> 1e-6 after five), so 1e-5 is asked
    tol = FP64_TOL if tag == "unit" else 1e-5
    assert rel(X1, g[f"redist1_{tag}"]) < tol
    assert rel(X5, g[f"redist5_{tag}"]) < tol
    assert rel(oc.alignCenterAngle(T(X), T(g[f"redist5_{tag}"])), g[f"align_{tag}"]) < FP64_TOL
    Xc = oc.correctAreaAndLengthAugLag(T(g[f"pert_{tag}"]), T(g[f"a0_{tag}"]), T(g[f"l0_{tag}"]))
    assert rel(Xc, g[f"corrected_{tag}"]) < 1e-9


def test_near_sing_int_rbf_matches_reference(golden):
    """nearSingInt_rbf on the device against the reference (golden rbf_fp64):
    FP64 all-pairs sums, FP64 RBF fits of the vesicles that have near pairs."""
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.filter import interpft_vec
    from ves2dpy_gb300.poten import Poten
    g = golden("rbf_fp64")
    for tag, N in (("n32", 32), ("n128", 128)):
        X = T(g[f"X_{tag}"])
        nv = X.shape[1]
        ves = capsules(X, None, None, 1.0, torch.ones(nv))
        op = Poten(N)
        G = op.stokesSLmatrix(ves, "fp64")
        near = naiveNearZoneInfo(X, interpft_vec(X, op.Nup))
        SLP = lambda F: op.exactStokesSLdiag(ves, G, F)  # noqa: E731
        LP = op.nearSingInt_rbf(ves, T(g[f"f_{tag}"]), SLP, near, None, ves, True, precision="fp64")
        assert rel(LP, g[f"LP_{tag}"]) < 1e-10, (tag, rel(LP, g[f"LP_{tag}"]))
        # the correction is a large part of the result on these packed clusters
        assert rel(g[f"far_{tag}"], g[f"LP_{tag}"]) > 1e-2


def test_time_step_near_rbf_fp64(golden):
    """The BIEM step with the matvec near field by nearSingInt_rbf (the
    alternative at mytorch/tstep_biem.py:494, the newtorch stepper's choice)
    on the packed near cluster."""
    g = golden("step_near_rbf_fp64")
    Xn, sn, _, _, it, iflag = _step(g["X0"], float(g["dt"]), float(g["speed"]), near="py_rbf")
    assert not iflag and it == int(g["iter1"])
    assert rel(Xn, g["X1"]) < FP64_TOL, rel(Xn, g["X1"])
    assert rel(sn, g["sig1"]) < 1e-8, rel(sn, g["sig1"])


def test_time_step_with_repulsion_fp64(golden):
    """The BIEM step with repulsion (tstep_biem.py:250-264): penalty force on
    the current shapes, G rep + nearSingInt_rbf(rep) added to the position
    right-hand side; matvec near field nearSingInt_hh."""
    from ves2dpy_gb300.tstep_biem import TStepBiem
    g = golden("step_rep_fp64")
    X = g["X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=float(g["dt"]), kappa=1.0, gmresTol=1e-10, gmresMaxIter=200, farFieldSpeed=float(g["speed"]),
                 viscCont=[1.0] * nv, repStrength=float(g["W"]), minDist=float(g["eta"]))
    options = dict(farField="shear", usePreco=True, repulsion=True)
    tt = TStepBiem(T(X), None, options, prams, near="py_hh", farfield_precision="fp64", sl_precision="fp64")
    Xn, sn, _, _, it, iflag = tt.time_step(T(X), torch.zeros(N, nv, dtype=torch.float64, device=dev()))
    assert not iflag and it == int(g["iter1"])
    assert rel(Xn, g["X1"]) < FP64_TOL, rel(Xn, g["X1"])
    assert rel(sn, g["sig1"]) < 1e-8, rel(sn, g["sig1"])


def test_bg_flow(golden):
    """ves_bg_flow against the reference's bg_flow (mytorch/tstep_biem.py:849-952)
    for every unconfined kind, with non-default speed, width and vortex size."""
    from ves2dpy_gb300.tstep_biem import TStepBiem
    g = golden("bgflow_fp64")
    X = g["X"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=1e-4, kappa=1.0, gmresTol=1e-10, gmresMaxIter=100, farFieldSpeed=1.0, viscCont=[1.0] * nv)
    tt = TStepBiem(T(X), None, dict(farField="shear", usePreco=True), prams)
    for kind in g["kinds"]:
        v = tt.bg_flow(T(X), None, str(kind), Speed=1.7, chanWidth=2.3, vortexSize=1.9)
        assert rel(v, g[f"v_{kind}"]) < 1e-14, kind


@pytest.mark.parametrize("ff", ["fp64", "fp32m"])
def test_fp32_preconditioner_gives_the_fp64_preconditioned_step(golden, ff):
    """The block-diagonal preconditioner built and factored in FP32 (the FP64
    system is still what GMRES solves): the step's result within GMRES's
    tolerance of the FP64-preconditioned step's, at most two more matvecs."""
    from ves2dpy_gb300.tstep_biem import TStepBiem
    g = golden("step_c1_fp64")
    X = g["X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    tol = 1e-10 if ff == "fp64" else 1e-8
    prams = dict(dt=float(g["dt"]), kappa=1.0, gmresTol=tol, gmresMaxIter=200, farFieldSpeed=float(g["speed"]),
                 viscCont=[1.0] * nv)
    out = {}
    for pp in ("fp64", "fp32"):
        tt = TStepBiem(T(X), None, dict(farField="shear", usePreco=True), prams, farfield_precision=ff,
                       sl_precision="fp64" if ff == "fp64" else "fp32c", precond_precision=pp)
        Xn, sn, _, _, it, iflag = tt.time_step(T(X), torch.zeros(N, nv, dtype=torch.float64, device=dev()))
        assert not iflag
        out[pp] = (Xn.cpu().numpy(), it)
    assert rel(out["fp32"][0], out["fp64"][0]) < 10 * tol
    assert out["fp32"][1] <= out["fp64"][1] + 2, (out["fp32"][1], out["fp64"][1])
