"""Double layer of vesicles with a viscosity contrast on the device against
the reference (golden dl_fp64) and, with near pairs, the FP64 oracle.

Tolerances (relative, max-norm): FP64 1e-10; the D matrix with its
restriction products in FP32 1e-5."""
import numpy as np
import pytest
import torch

from oracle import ves2d_oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def dev():
    return torch.device("cuda:0")


def T(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device=dev())


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("tag", ["n32", "n128"])
def test_stokes_dl_matrix_and_diag(golden, tag):
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    g = golden("dl_fp64")
    X, visc, f = g[f"X_{tag}"], g[f"visc_{tag}"], g[f"f_{tag}"]
    N = X.shape[0] // 2
    ves = capsules(T(X), None, None, 1.0, torch.tensor(visc))
    op = Poten(N)
    D = op.stokesDLmatrix(ves)
    assert rel(D, g[f"D_{tag}"]) < FP64_TOL, rel(D, g[f"D_{tag}"])
    for k, v in enumerate(visc):
        if v == 1:
            assert bool(torch.all(D[:, :, k] == 0))
    assert rel(op.exactStokesDLdiag(ves, D, T(f)), g[f"DLdiag_{tag}"]) < FP64_TOL
    D32 = op.stokesDLmatrix(ves, precision="fp32c")
    assert rel(D32, g[f"D_{tag}"]) < 1e-5, rel(D32, g[f"D_{tag}"])


@pytest.mark.parametrize("tag", ["n32", "n128"])
def test_exact_stokes_dl_and_far_field(golden, tag):
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    g = golden("dl_fp64")
    X, visc, f = g[f"X_{tag}"], g[f"visc_{tag}"], g[f"f_{tag}"]
    N, nv = X.shape[0] // 2, X.shape[1]
    ves = capsules(T(X), None, None, 1.0, torch.tensor(visc))
    op = Poten(N)
    dl = op.exactStokesDL(ves, T(f), T(g[f"Xtar_{tag}"]), list(range(nv)))
    assert rel(dl, g[f"DL_{tag}"]) < FP64_TOL, rel(dl, g[f"DL_{tag}"])
    # one target column, a subset of sources
    one = op.exactStokesDL(ves, T(f), T(g[f"Xtar_{tag}"][:, :1]), [nv - 1])
    sa, tang, _ = O.diff_prop(X)
    ref = O.exact_stokes_dl(X, tang, sa, f, visc, g[f"Xtar_{tag}"][:, :1], K1=[nv - 1])
    assert rel(one, ref) < FP64_TOL
    # nearSingInt with kernelDirect = exactStokesDL, as the step calls it (no near pairs here)
    D = op.stokesDLmatrix(ves)
    jump = 0.5 * (1 - torch.tensor(visc, device=dev()))
    DLP = lambda F: F * jump[None, :] + op.exactStokesDLdiag(ves, D, F)  # noqa: E731
    near = naiveNearZoneInfo(T(X), None)
    far = op.nearSingInt(ves, T(f), DLP, near, op.exactStokesDL, ves, True)
    assert rel(far, g[f"far_{tag}"]) < FP64_TOL, rel(far, g[f"far_{tag}"])
    far_m = op.nearSingInt(ves, T(f), DLP, ves.getZone(), op.exactStokesDL, ves, True)
    assert rel(far_m, g[f"far_{tag}"]) < FP64_TOL


@pytest.mark.parametrize("scheme", ["py_hh", "matlab"])
def test_near_sing_int_dl_with_near_pairs_vs_oracle(golden, scheme):
    """Packed cluster (near pairs at both thresholds): far field with the near
    pairs removed plus the py_hh gather or the MATLAB Lagrange extrapolation
    with the double layer at the Lagrange points."""
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    X = golden("far_fp64")["X"]
    N, nv = X.shape[0] // 2, X.shape[1]
    visc = np.array([2.0, 1.0, 0.5, 3.0, 1.5, 0.8])[:nv]
    f = np.random.default_rng(4).normal(size=(2 * N, nv))
    tab = O.PotenTables(N)
    Do = O.stokes_dl_matrix(X, visc, tab)
    vself = f * (0.5 * (1 - visc))[None, :] + O.exact_stokes_sl_diag(Do, f)
    ves = capsules(T(X), None, None, 1.0, torch.tensor(visc))
    op = Poten(N)
    D = op.stokesDLmatrix(ves)
    jump = 0.5 * (1 - torch.tensor(visc, device=dev()))
    DLP = lambda F: F * jump[None, :] + op.exactStokesDLdiag(ves, D, F)  # noqa: E731
    if scheme == "py_hh":
        near = O.naive_near_zone_info(X, O.interpft_vec(X, tab.Nup))
        assert len(near[3][0]) > 0
        ref = O.near_sing_int_dl(X, f, vself, visc, tab, "py_hh", near=near)
        got = op.nearSingInt(ves, T(f), DLP, naiveNearZoneInfo(T(X), None), op.exactStokesDL, ves, True)
    else:
        entries, h = O.get_zone(X)
        assert len(entries) > 0
        ref = O.near_sing_int_dl(X, f, vself, visc, tab, "matlab", entries=entries, h=h)
        got = op.nearSingInt(ves, T(f), DLP, ves.getZone(), op.exactStokesDL, ves, True)
    far = O.near_sing_int_dl(X, f, vself, visc, tab, "none")
    assert rel(far, ref) > 1e-6   # the correction changes the result
    assert rel(got, ref) < FP64_TOL, rel(got, ref)


def _dl_step(g, use_preco):
    from ves2dpy_gb300.tstep_biem import TStepBiem
    X = g["step_X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=float(g["step_dt"]), kappa=1.0, gmresTol=1e-10, gmresMaxIter=200,
                 farFieldSpeed=float(g["step_speed"]), viscCont=torch.tensor(g["step_visc"]))
    options = dict(farField="shear", usePreco=use_preco, repulsion=False)
    tt = TStepBiem(T(X), None, options, prams, near="py_hh", farfield_precision="fp64", sl_precision="fp64")
    return tt.time_step(T(X), torch.zeros(N, nv, dtype=torch.float64, device=dev()))


def test_time_step_viscosity_contrast_matches_reference(golden):
    """One BIEM step with contrasts 3, 1, 0.5 (alpha, D, Fdlp in the
    right-hand side and the matvec), unpreconditioned GMRES from zero as the
    reference's usePreco=False call.  About 600 unpreconditioned iterations
    amplify rounding differences: the restart cycle in which the residual
    test trips may differ by one (21 matvecs), and the tension, which the
    1e-10 residual pins less tightly than the positions, agrees to 1e-6."""
    g = golden("dl_fp64")
    Xn, sn, _, _, it, iflag = _dl_step(g, False)
    info = (it, int(g["step_iter1"]), rel(Xn, g["step_X1"]), rel(sn, g["step_sig1"]))
    assert not iflag, info
    assert rel(Xn, g["step_X1"]) < FP64_TOL, info
    assert rel(sn, g["step_sig1"]) < 1e-6, info
    assert abs(it - int(g["step_iter1"])) <= 21, info


def test_time_step_viscosity_contrast_preconditioned(golden):
    """The same step with the block preconditioner [I - D/alpha + dt kappa G
    Ben/alpha, -dt G Ten/alpha; Div, 0]: far fewer matvecs, same solution."""
    g = golden("dl_fp64")
    Xn, sn, _, _, it, iflag = _dl_step(g, True)
    assert not iflag and it < int(g["step_iter1"]) // 5, it
    assert rel(Xn, g["step_X1"]) < 1e-8, rel(Xn, g["step_X1"])


UNIT_AREA = 0.65 / (4 * np.pi)  # reduced area 0.65 at unit length


@pytest.mark.parametrize("nv,N,frac", [(256, 32, 0.2), (512, 128, 0.15)])
def test_double_layer_multipole_vs_direct(nv, N, frac):
    """exactStokesDL with the multipole series for separated pairs (FP32M)
    against the FP64 direct sum, for a random density and for the positions
    themselves (the density the step applies the operator to: a large mean
    that the double layer of a closed curve cancels).  Targets are other
    vesicles' points down to min_gap = 0.02 from a source, i.e. inside the
    near zone the step excludes; the FP32 tolerance of the far field, 1e-5."""
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    from ves2dpy_gb300.suspension import random_suspension
    X = random_suspension(nv, N, frac, min_gap=0.02, area=UNIT_AREA, seed=5)
    rng = np.random.default_rng(9)
    visc = rng.choice([0.5, 1.0, 3.0], size=nv)
    ves = capsules(T(X), None, None, 1.0, torch.tensor(visc))
    op = Poten(N)
    for f in (T(rng.normal(size=(2 * N, nv))), T(X)):
        # targets: 24 vesicles of the suspension, each against all the others
        got, ref = [], []
        for c in range(0, nv, nv // 24):
            K = [j for j in range(nv) if j != c]
            got.append(op.exactStokesDL(ves, f, ves.X[:, c:c + 1], K, precision="fp32m"))
            ref.append(op.exactStokesDL(ves, f, ves.X[:, c:c + 1], K))
        err = rel(torch.cat(got, 1), torch.cat(ref, 1).cpu().numpy())
        assert err < 1e-5, err


def test_near_sing_int_dl_multipole_with_near_pairs(golden):
    """nearSingInt with the double layer, FP32M far field vs FP64, on the
    packed cluster (near pairs: those pairs are summed directly in both)."""
    from ves2dpy_gb300.biem_support import naiveNearZoneInfo
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    X = golden("far_fp64")["X"]
    N, nv = X.shape[0] // 2, X.shape[1]
    visc = np.array([2.0, 1.0, 0.5, 3.0, 1.5, 0.8])[:nv]
    ves = capsules(T(X), None, None, 1.0, torch.tensor(visc))
    op = Poten(N)
    D = op.stokesDLmatrix(ves)
    jump = 0.5 * (1 - torch.tensor(visc, device=dev()))
    DLP = lambda F: F * jump[None, :] + op.exactStokesDLdiag(ves, D, F)  # noqa: E731
    near = naiveNearZoneInfo(T(X), None)
    for f in (T(np.random.default_rng(4).normal(size=(2 * N, nv))), T(X)):
        a = op.nearSingInt(ves, f, DLP, near, op.exactStokesDL, ves, True, precision="fp64")
        b = op.nearSingInt(ves, f, DLP, near, op.exactStokesDL, ves, True, precision="fp32m")
        assert rel(b, a.cpu().numpy()) < 1e-6, rel(b, a.cpu().numpy())


def test_time_step_viscosity_contrast_multipole(golden):
    """The contrast step with both far fields in FP32M (single layer and
    double layer) and the FP32 Alpert build, preconditioned, GMRES to 1e-8:
    positions within 1e-7 of the reference's FP64 step."""
    from ves2dpy_gb300.tstep_biem import TStepBiem
    g = golden("dl_fp64")
    X = g["step_X0"]
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=float(g["step_dt"]), kappa=1.0, gmresTol=1e-8, gmresMaxIter=200,
                 farFieldSpeed=float(g["step_speed"]), viscCont=torch.tensor(g["step_visc"]))
    options = dict(farField="shear", usePreco=True, repulsion=False)
    tt = TStepBiem(T(X), None, options, prams, near="py_hh", farfield_precision="fp32m", sl_precision="fp32c")
    Xn, sn, _, _, it, iflag = tt.time_step(T(X), torch.zeros(N, nv, dtype=torch.float64, device=dev()))
    assert not iflag
    assert rel(Xn, g["step_X1"]) < 1e-7, rel(Xn, g["step_X1"])
