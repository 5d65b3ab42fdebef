"""Suspensions of several point counts, CPU side.

The oracle's multi-group step (every vesicle of every group in one GMRES
system, MATLAB near rules between groups with the source group's h) must
reduce to the single-N step when the groups share N: the same suspension
split into two groups gives the same step.  For equal near-zone widths both
groups hold a vesicle of the minimum length (a far copy of the shortest one).
"""
import numpy as np

from oracle import ves2d_oracle as O


def small_suspension(N=16, nv=5, seed=1):
    from ves2dpy_gb300.suspension import vesicle_shape
    rng = np.random.default_rng(seed)
    X = np.zeros((2 * N, nv))
    for k in range(nv):
        x, y = vesicle_shape(N, rng, 0.8, area=0.06)
        X[:N, k] = x + (k % 3) * 0.32
        X[N:, k] = y + (k // 3) * 0.30
    return X


def split_with_shortest(X, cut):
    """Groups X[:, :cut] and X[:, cut:], the group without the shortest
    vesicle extended by a copy of it moved far away."""
    N = X.shape[0] // 2
    k = int(np.argmin(O.geom_prop(X)[2]))
    far = X[:, k:k + 1].copy()
    far[:N] += 40.0
    A, B = X[:, :cut], X[:, cut:]
    if k < cut:
        B = np.concatenate([B, far], axis=1)
    else:
        A = np.concatenate([A, far], axis=1)
    return A, B


def test_mixed_oracle_reduces_to_single_n():
    X = small_suspension()
    A, B = split_with_shortest(X, 2)
    U = np.concatenate([A, B], axis=1)
    N = X.shape[0] // 2
    prm = O.StepParams(dt=1e-4, speed=2.0, near="matlab")
    ref = O.time_step(U, np.zeros((N, U.shape[1])), prm)
    Xo, so, it, info = O.time_step_mixed([A, B], [np.zeros((N, A.shape[1])), np.zeros((N, B.shape[1]))], prm)
    assert info == 0 and it == ref.iters
    Xm = np.concatenate(Xo, axis=1)
    sm = np.concatenate(so, axis=1)
    assert np.abs(Xm - ref.X).max() < 1e-12 * np.abs(ref.X).max()
    assert np.abs(sm - ref.sigma).max() < 1e-9 * np.abs(ref.sigma).max()


def test_cross_zone_matches_single_set_zone():
    """Entries between two subsets = the single-set zone's entries between them."""
    X = small_suspension(nv=6, seed=3)
    N = X.shape[0] // 2
    ent, h = O.get_zone(X)
    src, tar = [0, 2, 4], [1, 3, 5]
    cross = O.get_zone_cross(X[:, src], X[:, tar], h)
    want = sorted((src.index(e.k1), tar.index(e.k2), e.j, e.icp) for e in ent if e.k1 in src and e.k2 in tar)
    got = sorted((e.k1, e.k2, e.j, e.icp) for e in cross)
    assert got == want and len(got) > 0


def test_mixed_step_argument_checks():
    """Host-side checks of the multi-group stepper (no device needed)."""
    import ctypes

    import pytest

    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.tstep_biem import TStepBiemMixed
    X = small_suspension()
    prams = dict(dt=1e-4, kappa=1.0, gmresTol=1e-10, gmresMaxIter=200)
    with pytest.raises(NotImplementedError):
        TStepBiemMixed([X, X], {}, prams, near="py_hh")
    with pytest.raises(ValueError):
        TStepBiemMixed([X] * 5, {}, prams)
    with pytest.raises(NotImplementedError):
        TStepBiemMixed([X, X], {"repulsion": True}, prams)
    # the C entry point rejects a bad group count without touching a device
    lib = nat.load_library()
    p = nat.StepParams()
    assert lib.ves_biem_step_mixed_workspace(0, None, ctypes.byref(p), None) == 0
    assert lib.ves_biem_step_mixed_workspace(5, None, ctypes.byref(p), None) == 0


def test_mixed_suspension_generator():
    """Groups keep their point counts; every pair of curves keeps the gap;
    centres lie in the rectangle sized for the area fraction; the reduced
    areas spread over the requested range."""
    import math

    from ves2dpy_gb300.suspension import mixed_suspension
    groups = [(24, 16), (6, 32)]
    Xs = mixed_suspension(groups, 0.2, box_aspect=2.0, min_gap=0.05, reduced_area=(0.6, 0.9), seed=3)
    assert [X.shape for X in Xs] == [(2 * N, nv) for nv, N in groups]
    curves = [(X[: X.shape[0] // 2, k], X[X.shape[0] // 2:, k]) for X in Xs for k in range(X.shape[1])]
    gap = min(np.sqrt(((xa[:, None] - xb[None, :]) ** 2 + (ya[:, None] - yb[None, :]) ** 2).min())
              for i, (xa, ya) in enumerate(curves) for (xb, yb) in curves[i + 1:])
    assert gap >= 0.05
    Ly = math.sqrt(30 * math.pi / 0.2 / 2.0)
    cy = np.array([c[1].mean() for c in curves])
    assert np.abs(cy).max() <= 0.5 * Ly + 2.0
    # base ellipses drawn with reduced areas in [0.6, 0.9]; the k = 2..8
    # perturbation moves the measured value by a few hundredths
    ra = np.concatenate([O.geom_prop(X)[0] for X in Xs])
    assert np.ptp(ra) > 0.2 and ra.min() > 0.45 and ra.max() < 1.0


def test_mixed_oracle_three_groups_reduce_to_single_n():
    """Three one-N groups (each holding a vesicle of the minimum length) give the single-N step."""
    X = small_suspension(nv=5, seed=1)
    N = X.shape[0] // 2
    k = int(np.argmin(O.geom_prop(X)[2]))
    groups = [X[:, :2], X[:, 2:4], X[:, 4:]]
    for g in range(3):
        if not any(np.array_equal(X[:, k], groups[g][:, j]) for j in range(groups[g].shape[1])):
            far = X[:, k:k + 1].copy()
            far[:N] += 40.0 * (g + 1)
            groups[g] = np.concatenate([groups[g], far], axis=1)
    U = np.concatenate(groups, axis=1)
    prm = O.StepParams(dt=1e-4, speed=2.0, near="matlab")
    ref = O.time_step(U, np.zeros((N, U.shape[1])), prm)
    Xo, so, it, info = O.time_step_mixed(groups, [np.zeros((N, G.shape[1])) for G in groups], prm)
    assert info == 0 and it == ref.iters
    assert np.abs(np.concatenate(Xo, axis=1) - ref.X).max() < 1e-12 * np.abs(ref.X).max()
