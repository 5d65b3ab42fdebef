"""Suspensions of several point counts on the GPU (ves_biem_step_mixed,
TStepBiemMixed).

* Groups of one N: the step equals the single-N step on the joined
  suspension (MATLAB near rules, FP64), both groups holding a vesicle of the
  minimum length so that their near-zone widths agree.
* Groups of N = 16 and N = 32 close enough for near pairs inside and between
  the groups: against the oracle's multi-group step at 1e-9, the tolerance of
  the MATLAB-scheme step test.
* The multipole precision (one all-pairs launch over every group) against
  the FP64 per-pair step of the same suspension.
* The uneven suspension (3000 vesicles of N = 32 and 1000 of N = 128, reduced
  areas uniform in [0.6, 0.9], 20% area fraction, Poiseuille flow
  u = (1 - y^2 / W^2, 0) with W = 60): GMRES converges at 1e-8 with the FP32
  far field and the step commutes with a translation along the channel.
"""
import math

import numpy as np
import pytest
import torch

from oracle import ves2d_oracle as O
from test_mixed import small_suspension, split_with_shortest

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def T(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device=DEV)


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


PRAMS = dict(dt=1e-4, kappa=1.0, gmresTol=1e-10, gmresMaxIter=200, farFieldSpeed=2.0, viscCont=1.0)
OPTS = dict(farField="shear", usePreco=True, repulsion=False)


def test_mixed_same_n_matches_single_step():
    from ves2dpy_gb300.tstep_biem import TStepBiem, TStepBiemMixed
    X = small_suspension()
    A, B = split_with_shortest(X, 2)
    U = np.concatenate([A, B], axis=1)
    N = X.shape[0] // 2
    one = TStepBiem(T(U), None, OPTS, PRAMS, near="matlab", farfield_precision="fp64", sl_precision="fp64")
    Xr, sr, _, _, it_r, fl_r = one.time_step(T(U), torch.zeros(N, U.shape[1], dtype=torch.float64, device=DEV))
    mix = TStepBiemMixed([T(A), T(B)], OPTS, PRAMS, near="matlab", farfield_precision="fp64", sl_precision="fp64")
    Xo, so, it, fl = mix.time_step([T(A), T(B)], [torch.zeros(N, A.shape[1], dtype=torch.float64, device=DEV),
                                                  torch.zeros(N, B.shape[1], dtype=torch.float64, device=DEV)])
    assert not fl and not fl_r and it == it_r
    assert mix.last.n_near_entries == one.last.n_near_entries > 0
    assert rel(torch.cat(Xo, 1), Xr) < 1e-12
    assert rel(torch.cat(so, 1), sr) < 1e-9


def _two_sizes():
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(5)
    groups = []
    for N, nv, x0 in ((16, 3, 0.0), (32, 2, 0.16)):
        X = np.zeros((2 * N, nv))
        for k in range(nv):
            x, y = vesicle_shape(N, rng, 0.8, area=0.06)
            X[:N, k] = x + x0 + k * 0.32
            X[N:, k] = y + (0.0 if N == 16 else 0.30)
        groups.append(X)
    return groups


def test_mixed_two_sizes_vs_oracle():
    from ves2dpy_gb300.tstep_biem import TStepBiemMixed
    Xs = _two_sizes()
    hs = [O.geom_prop(X)[2].min() / (X.shape[0] // 2) for X in Xs]
    cross = len(O.get_zone_cross(Xs[1], Xs[0], hs[1])) + len(O.get_zone_cross(Xs[0], Xs[1], hs[0]))
    assert cross > 0, "the groups have near pairs between them"
    sig = [np.zeros((X.shape[0] // 2, X.shape[1])) for X in Xs]
    prm = O.StepParams(dt=1e-4, speed=2.0, near="matlab")
    ref_X, ref_s, ref_it, ref_info = O.time_step_mixed(Xs, sig, prm)
    mix = TStepBiemMixed([T(X) for X in Xs], OPTS, PRAMS, near="matlab", farfield_precision="fp64",
                         sl_precision="fp64")
    Xo, so, it, fl = mix.time_step([T(X) for X in Xs], [T(s) for s in sig])
    assert not fl and ref_info == 0
    assert abs(mix.last.matvecs - ref_it) <= 1
    for g in range(2):
        assert rel(Xo[g], ref_X[g]) < 1e-9, (g, rel(Xo[g], ref_X[g]))
        assert rel(so[g], ref_s[g]) < 1e-6, (g, rel(so[g], ref_s[g]))



def test_mixed_fp32m_one_launch_matches_fp64():
    """With the multipole precision the far field of every group from the
    sources of every group runs as one launch (farfield_mp_groups_run), and
    the MATLAB corrections per pair of groups follow; the step agrees with the
    FP64 step that sums group pair by group pair, to the FP32 accuracy of the
    sums: velocities (Xnew - X)/dt at 1e-5, GMRES counts within one."""
    from ves2dpy_gb300.tstep_biem import TStepBiemMixed
    Xs = _two_sizes()
    sig = [torch.zeros(X.shape[0] // 2, X.shape[1], dtype=torch.float64, device=DEV) for X in Xs]
    prams = dict(PRAMS, gmresTol=1e-8)
    out = {}
    for prec in ("fp64", "fp32m"):
        mix = TStepBiemMixed([T(X) for X in Xs], OPTS, prams, near="matlab", farfield_precision=prec,
                             sl_precision="fp64")
        Xo, so, it, fl = mix.time_step([T(X) for X in Xs], sig)
        assert not fl
        out[prec] = (Xo, mix.last.matvecs)
    for g in range(2):
        v64 = (out["fp64"][0][g] - T(Xs[g])) / PRAMS["dt"]
        v32 = (out["fp32m"][0][g] - T(Xs[g])) / PRAMS["dt"]
        assert rel(v32, v64) < 1e-5, (g, rel(v32, v64))
    assert abs(out["fp32m"][1] - out["fp64"][1]) <= 1

def test_uneven_suspension_poiseuille():
    from ves2dpy_gb300.suspension import mixed_suspension
    from ves2dpy_gb300.tstep_biem import TStepBiemMixed
    W = 60.0
    Xs = mixed_suspension([(3000, 32), (1000, 128)], 0.20, box_aspect=5.0, min_gap=0.1, reduced_area=(0.6, 0.9),
                          seed=0)
    assert max(np.abs(X[X.shape[0] // 2:]).max() for X in Xs) < W
    prams = dict(dt=1e-5, kappa=1.0, gmresTol=1e-8, gmresMaxIter=200, farFieldSpeed=1.0, chanWidth=W, viscCont=1.0)
    opts = dict(farField="parabolic", usePreco=True, repulsion=False)
    sig = [torch.zeros(X.shape[0] // 2, X.shape[1], dtype=torch.float64, device=DEV) for X in Xs]
    out = []
    for dx in (0.0, 7.5):
        Xg = [T(X) for X in Xs]
        for X in Xg:
            X[: X.shape[0] // 2] += dx
        mix = TStepBiemMixed(Xg, opts, prams, near="matlab", farfield_precision="fp32m", sl_precision="fp32c")
        Xo, so, it, fl = mix.time_step(Xg, sig)
        assert not fl and mix.last.resid <= 1e-8, (it, mix.last.resid)
        assert mix.last.n_near_entries > 0
        out.append((Xg, Xo, so))
    (X0, Xa, sa), (X1, Xb, sb) = out
    for g in range(2):
        disp = Xa[g] - X0[g]
        assert float(disp.abs().max()) > 0
        moved = Xb[g].clone()
        moved[: moved.shape[0] // 2] -= 7.5
        assert float((moved - Xa[g]).abs().max()) < 1e-3 * float(disp.abs().max())
        assert rel(sb[g], sa[g]) < 1e-4, rel(sb[g], sa[g])
