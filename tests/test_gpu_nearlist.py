"""Near-pair candidate lists built on the device (the bucket-sorted search of
ves_near.cu) against a brute-force bounding-box test, their capacity growth,
and the handling of a non-finite shape.

The reference's naiveNearZoneInfo (mytorch/biem_support.py:520-613) keeps
every pair and has no capacity; the device lists have one, report the count
they need, and the Python layer re-runs the build (or the whole step, whose
inputs are unchanged) with room for it.  A NaN coordinate raises instead of
making its vesicle a near pair of every other one.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def _boxes(X):
    N = X.shape[0] // 2
    return np.stack([X[:N].min(0), X[:N].max(0), X[N:].min(0), X[N:].max(0)], axis=1)


def _brute_lists(X, Xup, thr):
    """For every target vesicle, the other vesicles whose upsampled box comes
    closer than thr to its coarse box (Euclidean box gap)."""
    tb, sb = _boxes(X), _boxes(Xup)
    gx = np.maximum(0.0, np.maximum(sb[None, :, 0] - tb[:, None, 1], tb[:, None, 0] - sb[None, :, 1]))
    gy = np.maximum(0.0, np.maximum(sb[None, :, 2] - tb[:, None, 3], tb[:, None, 2] - sb[None, :, 3]))
    hit = gx * gx + gy * gy < thr * thr
    np.fill_diagonal(hit, False)
    return [np.nonzero(hit[t])[0] for t in range(X.shape[1])]


def _device_lists(nz):
    cnt = nz.cand_count.cpu().numpy()[: nz.nv]
    src = nz.cand_src.cpu().numpy()[: nz.nv * nz.maxc].reshape(nz.nv, nz.maxc)
    return [src[t, : cnt[t]] for t in range(nz.nv)]


def _build(X, thr=0.0, maxc=32):
    from oracle import ves2d_oracle as O
    from ves2dpy_gb300.biem_support import NearZone
    from ves2dpy_gb300.layout import to_vm
    N = X.shape[0] // 2
    Xup = O.interpft_vec(X, N * int(np.ceil(np.sqrt(N))))
    Xt = torch.tensor(X, dtype=torch.float64, device=DEV)
    Xupt = torch.tensor(Xup, dtype=torch.float64, device=DEV)
    nz = NearZone.build_py(to_vm(Xt), N, to_vm(Xupt), thr, maxc=maxc)
    return nz, Xup


@pytest.mark.parametrize("case", ["random", "outlier", "wide_threshold"])
def test_grid_candidates_match_brute_force(case):
    from ves2dpy_gb300.suspension import lattice_suspension, random_suspension
    if case == "random":
        X, thr = random_suspension(1500, 32, 0.2, min_gap=0.05, seed=3), 0.0
    elif case == "outlier":
        # one vesicle far from the rest stretches the grid's extent
        X = random_suspension(400, 32, 0.2, min_gap=0.05, seed=4)
        X[:32, 7] += 1.0e5
        thr = 0.0
    else:
        # a threshold of several spacings: > 100 candidates per vesicle, more
        # than the initial capacity of 32, so the build has to grow
        X, thr = lattice_suspension(14, 32, spacing=3.0, jitter=0.2, min_gap=0.3, seed=5), 18.0
    N = X.shape[0] // 2
    nz, Xup = _build(X, thr)
    want = _brute_lists(X, Xup, thr if thr > 0 else 1.0 / N)
    got = _device_lists(nz)
    for t in range(X.shape[1]):
        np.testing.assert_array_equal(got[t], want[t], err_msg=f"target vesicle {t}")
    if case == "wide_threshold":
        assert max(len(w) for w in want) > 100 and nz.maxc >= max(len(w) for w in want)


def test_capacity_growth_gives_the_same_exclusions():
    """A build that starts too small and grows equals one sized right from the start."""
    from ves2dpy_gb300.suspension import lattice_suspension
    X = lattice_suspension(10, 32, spacing=2.4, jitter=0.1, min_gap=0.05, seed=6)
    small, _ = _build(X, 6.0, maxc=2)
    big, _ = _build(X, 6.0, maxc=1024)
    assert small.maxc < big.maxc
    for a, b in zip(small.ids(), big.ids()):
        np.testing.assert_array_equal(a, b)


def test_nonfinite_shape_raises_instead_of_overflowing():
    from ves2dpy_gb300.suspension import random_suspension
    X = random_suspension(300, 32, 0.2, min_gap=0.05, seed=7)
    X[5, 123] = np.nan
    with pytest.raises(ValueError, match="vesicle 123 has a non-finite coordinate"):
        _build(X)


def test_biem_step_grows_its_lists():
    """The BIEM step re-runs with a larger capacity when its lists overflow,
    and gives the result of a run whose capacity was large enough."""
    from ves2dpy_gb300.suspension import lattice_suspension
    from ves2dpy_gb300.tstep_biem import TStepBiem
    X = lattice_suspension(6, 32, spacing=2.6, jitter=0.05, min_gap=0.03, seed=8)
    N, nv = X.shape[0] // 2, X.shape[1]
    prams = dict(dt=1e-4, kappa=1.0, gmresTol=1e-10, gmresMaxIter=100, farFieldSpeed=2.0, viscCont=[1.0] * nv)
    opts = dict(farField="shear", usePreco=True, repulsion=False)
    Xt = torch.tensor(X, dtype=torch.float64, device=DEV)
    sig = torch.zeros(N, nv, dtype=torch.float64, device=DEV)
    out = []
    for maxc in (1, 512):
        tt = TStepBiem(Xt, None, opts, prams, near="py_hh", farfield_precision="fp64", sl_precision="fp64")
        tt._maxc = maxc
        Xn, sn, *_ = tt.time_step(Xt, sig)
        out.append((Xn.cpu().numpy(), sn.cpu().numpy(), tt._maxc))
    assert out[0][2] > 1
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
