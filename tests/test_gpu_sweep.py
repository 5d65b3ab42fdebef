"""Far-field + near-singular sweep: nv in {1024, 4096, 16384} x N in {32, 128}.

Vesicles of reduced area 0.65 and area pi (perturbation modes k = 2..8,
random rotation), centres uniform in a square sized for 20% area fraction,
rejection at min gap 0.05; random N(0, 1) FP64 densities per point; one
evaluation each.

* All-pairs sum with the exclusions of allExactStokesSLTarget_compare1
  (mytorch/biem_support.py:7-121, threshold length / N): the multipole path
  (fp32m) over every target column, the direct FP32C and FP64 rules on a
  block of columns.  fp32m and fp32c against fp64 at the FP32 far-field
  tolerance 1e-5; fp64 against the FP64 oracle (the same sum restated on the
  host, over the non-excluded sources) at 1e-10 on a few target points.
* Near-singular integration (MATLAB nearSingInt, matlab/poten_py.m:495-692,
  with the zones of getZone): at a few near target points the Lagrange part
  (FP64) against the oracle and the whole layer potential (fp32m far
  field) at 1e-5 of the field's magnitude.  The oracle works on the vesicles
  around the target (every near source lies within h of it) with the
  suspension's h, and sums the far field over all sources.  The near
  correction's FP64 rounding grows with the absolute coordinates: the oracle
  itself changes by 6e-10 to 9e-10 (relative) under a translation by
  30 or 60 and by 1e-8 under one by 450 (N = 128, 155 near entries), so the
  suspension is centred on the origin, the checked points are the near
  points closest to it and the Lagrange part is compared at 1e-9, as the
  MATLAB-scheme step is.
"""
import numpy as np
import pytest
import torch

from oracle import ves2d_oracle as O

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
FP64_TOL = 1e-10
FP64_NEAR_TOL = 1e-9   # the MATLAB near correction near the origin (see above)
FP32_TOL = 1e-5
SIZES = [(1024, 32), (1024, 128), (4096, 32), (4096, 128), (16384, 32), (16384, 128)]
BLOCK = 16     # target columns checked against the FP64 direct rule


def T(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64, device=DEV)


def rel(a, b, scale=None):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    s = np.abs(b).max() if scale is None else scale
    return float(np.abs(a - b).max() / s)


def _suspension(nv, N, seed):
    from ves2dpy_gb300.suspension import random_suspension
    return random_suspension(nv, N, 0.20, min_gap=0.05, seed=seed)


def _upsampled(X):
    """Xup and sa_up of capsules(interpft(X, Nup)) in the reference layout."""
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.layout import from_vm, to_vm
    N, nv = X.shape[0] // 2, X.shape[1]
    ctx = nat.context(N, DEV)
    Nup = ctx.Nup
    Xup = torch.empty(nv, 2 * Nup, dtype=torch.float64, device=DEV)
    sa = torch.empty(nv, Nup, dtype=torch.float64, device=DEV)
    nat.check(ctx.lib.ves_upsample_geometry(ctx.handle, nv, to_vm(X).data_ptr(), Xup.data_ptr(), sa.data_ptr(),
                                            None, None, nat.stream_ptr(DEV)), "upsample geometry")
    return from_vm(Xup), from_vm(sa)


def _oracle_point(Xup, sa, fup, x, y, skip):
    """FP64 oracle far field at one point over every source vesicle not in ``skip``."""
    nv = Xup.shape[1]
    K1 = np.setdiff1d(np.arange(nv), np.asarray(sorted(skip), dtype=np.int64))
    out = np.zeros(2)
    for c in range(0, len(K1), 2048):
        out += O.exact_stokes_sl_points(Xup, sa, fup, np.array([[x], [y]]), K1[c:c + 2048])[:, 0]
    return out


@pytest.mark.parametrize("nv,N", SIZES)
def test_sweep_far_field(nv, N):
    from ves2dpy_gb300.biem_support import allExactStokesSLTarget_compare1
    X = T(_suspension(nv, N, seed=0))
    Xup, sa = _upsampled(X)
    Nup = Xup.shape[0] // 2
    g = torch.Generator(device=DEV).manual_seed(nv + N)
    fup = torch.randn(2 * Nup, nv, dtype=torch.float64, device=DEV, generator=g)
    length = float(O.geom_prop(X[:, :1].cpu().numpy())[2][0])
    # all targets by the multipole path; a block of columns by the direct rules
    u_m, ids = allExactStokesSLTarget_compare1(Xup, sa, fup, X, length=length, precision="fp32m")
    assert torch.isfinite(u_m).all()
    k0 = nv // 2
    blk = X[:, k0:k0 + BLOCK]
    u_64, _ = allExactStokesSLTarget_compare1(Xup, sa, fup, blk, length=length, offset=k0, precision="fp64")
    u_32, _ = allExactStokesSLTarget_compare1(Xup, sa, fup, blk, length=length, offset=k0, precision="fp32c")
    assert rel(u_m[:, k0:k0 + BLOCK], u_64) < FP32_TOL, rel(u_m[:, k0:k0 + BLOCK], u_64)
    assert rel(u_32, u_64) < FP32_TOL, rel(u_32, u_64)
    # FP64 against the oracle at target points of the block, one with exclusions if any
    ids0, ids1, ids2 = [np.asarray(a) for a in ids]
    src = ids0 + (ids0 >= ids2)
    inblk = np.nonzero((ids2 >= k0) & (ids2 < k0 + BLOCK))[0]
    pts = [(k0, 0), (k0 + BLOCK - 1, N // 2)]
    if len(inblk):
        pts.append((int(ids2[inblk[0]]), int(ids1[inblk[0]])))
    Xn, Xupn, san, fn = X.cpu().numpy(), Xup.cpu().numpy(), sa.cpu().numpy(), fup.cpu().numpy()
    ref, got = [], []
    for t, i in pts:
        skip = {t} | set(src[(ids2 == t) & (ids1 == i)].tolist())
        ref.append(_oracle_point(Xupn, san, fn, Xn[i, t], Xn[i + N, t], skip))
        got.append(u_64[[i, i + N], t - k0].cpu().numpy())
    assert rel(np.array(got), np.array(ref), np.abs(u_64.cpu().numpy()).max()) < FP64_TOL


@pytest.mark.parametrize("nv,N", SIZES)
def test_sweep_near_singular(nv, N):
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.poten import Poten
    Xn = _suspension(nv, N, seed=1)
    # centre the square on the origin (the near correction's rounding grows with |x|)
    Xn[:N] -= np.round(0.5 * (Xn[:N].min() + Xn[:N].max()))
    Xn[N:] -= np.round(0.5 * (Xn[N:].min() + Xn[N:].max()))
    X = T(Xn)
    g = torch.Generator(device=DEV).manual_seed(7 * nv + N)
    f = torch.randn(2 * N, nv, dtype=torch.float64, device=DEV, generator=g)
    ves = capsules(X, None, None, 1.0, 1.0)
    op = Poten(N)
    nz = ves.getZone()
    ids0, ids1, ids2 = nz.ids()
    assert len(ids0) > 0, "the sweep suspension has near pairs"
    src = ids0 + (ids0 >= ids2)
    h = nz.h
    # three near target points on the vesicles nearest the origin, and the
    # vesicles around them: every near source of a point lies within h of it
    cen = np.stack([Xn[:N].mean(0), Xn[N:].mean(0)], 1)
    picks = []
    for k in np.argsort(np.hypot(cen[ids2, 0], cen[ids2, 1]), kind="stable"):
        if (int(ids2[k]), int(ids1[k])) not in picks and int(ids2[k]) not in [p[0] for p in picks]:
            picks.append((int(ids2[k]), int(ids1[k])))
        if len(picks) == 3:
            break
    rmax = float(np.hypot(Xn[:N] - cen[:, 0], Xn[N:] - cen[:, 1]).max())
    locs = {t: np.nonzero(np.hypot(cen[:, 0] - cen[t, 0], cen[:, 1] - cen[t, 1]) <= 2 * rmax + 2 * h)[0]
            for t, _ in picks}
    # vself = G f: the FP64 Alpert matrix on those vesicles, the mixed-precision one elsewhere
    sub = torch.as_tensor(np.unique(np.concatenate(list(locs.values()))), device=DEV)
    vself = op.exactStokesSLdiag(ves, op.stokesSLmatrix(ves, "fp32c"), f)
    ves_sub = capsules(X[:, sub], None, None, 1.0, 1.0)
    vself[:, sub] = op.exactStokesSLdiag(ves_sub, op.stokesSLmatrix(ves_sub, "fp64"), f[:, sub])
    LP, near = op._near_common("matlab", ves, f, lambda F: vself, nz, "fp32m")
    assert torch.isfinite(LP).all()
    fn = f.cpu().numpy()
    Xup_all = O.interpft_vec(Xn, O.upsample_factor(N))
    fup_all = O.interpft_vec(fn, O.upsample_factor(N))
    sa_all = O.diff_prop(Xup_all)[0]
    tab = O.PotenTables(N)
    scale = float(LP.abs().max())
    lag_ref, lag_got, lp_ref, lp_got = [], [], [], []
    for t, i in picks:
        loc = locs[t]
        q = int(np.nonzero(loc == t)[0][0])
        Xl, fl = Xn[:, loc], fn[:, loc]
        vs_l = O.exact_stokes_sl_diag(O.stokes_sl_matrix(Xl, tab), fl)
        ent, _ = O.get_zone(Xl, h)
        near_l = [e.k1 for e in ent if e.k2 == q and e.j == i]
        assert sorted(int(loc[k]) for k in near_l) == sorted(src[(ids2 == t) & (ids1 == i)].tolist())
        Xupl, fupl = Xup_all[:, loc], fup_all[:, loc]
        sal = sa_all[:, loc]
        full_l = O.near_sing_int_matlab(Xl, fl, vs_l, ent, h, tab)
        far_l = O.all_exact_stokes_sl_target(Xupl, sal, fupl, Xl, None)
        corr = (full_l - far_l)[[i, i + N], q]      # sum over near sources of (Lagrange - trapezoid)
        trap = O.exact_stokes_sl_points(Xupl, sal, fupl, np.array([[Xn[i, t]], [Xn[i + N, t]]]), near_l)[:, 0]
        lag_ref.append(corr + trap)
        lag_got.append(near[[i, i + N], t].cpu().numpy())
        lp_ref.append(_oracle_point(Xup_all, sa_all, fup_all, Xn[i, t], Xn[i + N, t], {t}) + corr)
        lp_got.append(LP[[i, i + N], t].cpu().numpy())
    lag_ref, lag_got = np.array(lag_ref), np.array(lag_got)
    assert rel(lag_got, lag_ref) < FP64_NEAR_TOL, rel(lag_got, lag_ref)
    assert rel(np.array(lp_got), np.array(lp_ref), scale) < FP32_TOL, rel(np.array(lp_got), np.array(lp_ref), scale)
