"""Size-independent properties at the benchmark size, where the FP64 oracle
cannot run: the suspension of bench.py (4096 unit-length vesicles of reduced
area 0.65, N = 128, Nup = 1536, 15% area fraction, seed 0).

* all-pairs sum: the multipole path (fp32m) against the direct FP32C rule on
  a block of target columns (the FP32 far-field tolerance, 1e-5), linearity
  in the density and invariance under a translation of every point;
* BIEM step: GMRES converges at the bench tolerance and the step commutes
  with a translation along the flow (the shear (2y, 0) does not depend on x).

And the large-suspension case: 16384 vesicles of N = 32 (reduced area 0.65,
area fraction 25%, centres in [0, 32 pi]^2) in the Taylor-Green flow
u = (sin x cos y, -cos x sin y): the BIEM step converges and commutes with a
translation by one period (2 pi, 0) of the flow.
"""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu

NV, N = 4096, 128
UNIT_AREA = 0.65 / (4 * math.pi)
MIN_GAP = 0.05 / 7.79


@pytest.fixture(scope="module")
def susp():
    from ves2dpy_gb300.suspension import random_suspension
    X = random_suspension(NV, N, 0.15, min_gap=MIN_GAP, area=UNIT_AREA, seed=0)
    return torch.tensor(X, dtype=torch.float64, device="cuda:0")


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_allpairs_fullsize(susp):
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.biem_support import allExactStokesSLTarget_compare2
    from ves2dpy_gb300.layout import from_vm, to_vm
    from ves2dpy_gb300.poten import Poten
    op = Poten(N)
    X = susp
    # the upsampled curve and its jacobian (interpft_vec and capsules(Xup).sa)
    ctx = nat.context(N, X.device)
    Xup_v = torch.empty(NV, 2 * op.Nup, dtype=torch.float64, device=X.device)
    sa_v = torch.empty(NV, op.Nup, dtype=torch.float64, device=X.device)
    Xv = to_vm(X)
    nat.check(ctx.lib.ves_upsample_geometry(ctx.handle, NV, Xv.data_ptr(), Xup_v.data_ptr(), sa_v.data_ptr(),
                                            None, None, nat.stream_ptr(X.device)), "upsample geometry")
    Xup, sa = from_vm(Xup_v), from_vm(sa_v)
    g = torch.Generator(device="cuda:0").manual_seed(3)
    f1 = torch.randn(2 * op.Nup, NV, dtype=torch.float64, device=X.device, generator=g)
    f2 = torch.randn(2 * op.Nup, NV, dtype=torch.float64, device=X.device, generator=g)
    e = torch.zeros(0, dtype=torch.long)

    def far(Xs, Xt, f, prec, offset=0):
        return allExactStokesSLTarget_compare2(Xs, sa, f, Xt, e, e, e, offset=offset, precision=prec)

    u1 = far(Xup, X, f1, "fp32m")
    assert torch.isfinite(u1).all()
    k0 = 1000
    ref = far(Xup, X[:, k0:k0 + 64], f1, "fp32c", offset=k0)
    assert rel(u1[:, k0:k0 + 64], ref) < 1e-5, rel(u1[:, k0:k0 + 64], ref)
    # linearity in the density
    u2 = far(Xup, X, f2, "fp32m")
    u12 = far(Xup, X, f1 + 2 * f2, "fp32m")
    assert rel(u12, u1 + 2 * u2) < 1e-5, rel(u12, u1 + 2 * u2)
    # translation of every point (the sum depends on differences only)
    shift = torch.tensor([3.7] * op.Nup + [-1.3] * op.Nup, dtype=torch.float64, device=X.device)[:, None]
    tshift = torch.tensor([3.7] * N + [-1.3] * N, dtype=torch.float64, device=X.device)[:, None]
    ut = far(Xup + shift, X + tshift, f1, "fp32m")
    assert rel(ut, u1) < 1e-5, rel(ut, u1)


def test_biem_step_fullsize_translation(susp):
    from ves2dpy_gb300.tstep_biem import TStepBiem
    X = susp
    prams = dict(dt=1e-5, kappa=1.0, gmresTol=1e-8, gmresMaxIter=200, farFieldSpeed=2.0, viscCont=1.0)
    options = dict(farField="shear", usePreco=True, repulsion=False)
    sig = torch.zeros(N, NV, dtype=torch.float64, device=X.device)
    shift = torch.tensor([5.0] * N + [0.0] * N, dtype=torch.float64, device=X.device)[:, None]
    out = []
    for Xs in (X, X + shift):
        tt = TStepBiem(Xs, None, options, prams, near="py_hh", farfield_precision="fp32m", sl_precision="fp32c")
        Xn, sn, _, _, it, iflag = tt.time_step(Xs, sig)
        assert not iflag and tt.last.resid <= 1e-8, (it, tt.last.resid)
        out.append((Xn, sn))
    (X0, s0), (X1, s1) = out
    disp = X0 - X
    # positions move by dt*|u| ~ 1e-5; their translated steps agree to a small
    # fraction of that displacement, tensions to 1e-4
    assert float((X1 - shift - X0).abs().max()) < 1e-3 * float(disp.abs().max())
    assert rel(s1, s0) < 1e-4, rel(s1, s0)


def test_biem_step_large_taylor_green():
    from ves2dpy_gb300.suspension import random_suspension
    from ves2dpy_gb300.tstep_biem import TStepBiem
    nv, n = 16384, 32
    side = 32 * math.pi
    area = 0.25 * side * side / nv
    Xn = random_suspension(nv, n, 0.25, min_gap=0.3 * math.sqrt(4 * math.pi * area / 0.65) / n, area=area, seed=2)
    X = torch.tensor(Xn, dtype=torch.float64, device="cuda:0")
    # bg_flow 'taylorGreen' is vortexSize * (sin, -cos)(pi x / vortexSize) ...: vortexSize pi, speed 1/pi
    prams = dict(dt=1e-5, kappa=1.0, gmresTol=1e-8, gmresMaxIter=200, farFieldSpeed=1.0 / math.pi,
                 vortexSize=math.pi, viscCont=1.0)
    options = dict(farField="taylorGreen", usePreco=True, repulsion=False)
    sig = torch.zeros(n, nv, dtype=torch.float64, device=X.device)
    shift = torch.tensor([2 * math.pi] * n + [0.0] * n, dtype=torch.float64, device=X.device)[:, None]
    out = []
    for Xs in (X, X + shift):
        tt = TStepBiem(Xs, None, options, prams, near="py_hh", farfield_precision="fp32m", sl_precision="fp32c")
        Xnew, snew, _, _, it, iflag = tt.time_step(Xs, sig)
        assert not iflag and tt.last.resid <= 1e-8, (it, tt.last.resid)
        assert torch.isfinite(Xnew).all()
        out.append((Xnew, snew))
    (X0, s0), (X1, s1) = out
    disp = X0 - X
    assert float(disp.abs().max()) > 0
    assert float((X1 - shift - X0).abs().max()) < 1e-3 * float(disp.abs().max())
    assert rel(s1, s0) < 1e-4, rel(s1, s0)
