"""Seeded synthetic vesicle suspensions.

The reference drivers load initial conditions from ``.mat`` files that are not
part of the reference tree (``mytorch/driver_confined.py:135``,
``newtorch/entry_driver_manyfreeSpaceVesicle_N128.py:95``).  These generators
produce suspensions with the shapes, sizes and area fractions of the
benchmark workloads instead.  Every vesicle is an ellipse of prescribed
reduced area and area, whose radius is perturbed by Fourier modes k=2..8 with
N(0, amp) amplitudes, randomly rotated, and placed without overlap.

Layout is the reference's: ``X[2N, nv]``, x-coordinates in rows 0..N-1, y in
rows N..2N-1, one column per vesicle, float64.
"""
from __future__ import annotations

import functools
import math

import numpy as np


@functools.lru_cache(maxsize=4096)
def _axis_ratio(reduced_area: float) -> float:
    """Axis ratio a/b of the ellipse with reduced area 4*pi*A/L^2 (bisection)."""
    t = np.arange(4096) * 2 * np.pi / 4096

    def ra(ratio):
        L = np.sum(np.sqrt((ratio * np.sin(t)) ** 2 + np.cos(t) ** 2)) * 2 * np.pi / 4096
        return 4 * np.pi * np.pi * ratio / L ** 2

    lo, hi = 1.0, 50.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if ra(mid) > reduced_area:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def ellipse_axes(reduced_area: float, area: float = math.pi):
    """Semi-axes (a >= b) of the ellipse with this reduced area and area A."""
    ratio = _axis_ratio(round(float(reduced_area), 6))
    b = math.sqrt(area / (math.pi * ratio))
    return ratio * b, b


def vesicle_shape(N: int, rng: np.random.Generator, reduced_area: float = 0.65,
                  area: float = math.pi, amp: float = 0.02, modes=range(2, 9)):
    """One perturbed ellipse centred at the origin with a random rotation.

    Returns (x[N], y[N]) ordered counter-clockwise.
    """
    a, b = ellipse_axes(reduced_area, area)
    th = np.arange(N) * 2 * np.pi / N
    pert = np.ones(N)
    for k in modes:
        c, s = rng.normal(0.0, amp, size=2)
        pert += c * np.cos(k * th) + s * np.sin(k * th)
    x = a * np.cos(th) * pert
    y = b * np.sin(th) * pert
    phi = rng.uniform(0.0, 2 * np.pi)
    cph, sph = math.cos(phi), math.sin(phi)
    return cph * x - sph * y, sph * x + cph * y


def _min_gap(xa, ya, xb, yb):
    d2 = (xa[:, None] - xb[None, :]) ** 2 + (ya[:, None] - yb[None, :]) ** 2
    return math.sqrt(float(d2.min()))


def lattice_suspension(nv_side: int = 4, N: int = 32, spacing: float = 3.0, jitter: float = 0.1,
                       min_gap: float = 0.3, reduced_area: float = 0.65, seed: int = 0,
                       max_tries: int = 10000):
    """Vesicles on a jittered nv_side x nv_side lattice (sites in row-major order).

    A vesicle whose shape, rotation or jitter would come closer than
    ``min_gap`` to an already placed one is re-drawn (shape, rotation and
    jitter together), in placement order, until it fits.
    """
    rng = np.random.default_rng(seed)
    nv = nv_side * nv_side
    X = np.zeros((2 * N, nv))
    placed = []
    for k in range(nv):
        cx0 = (k % nv_side) * spacing
        cy0 = (k // nv_side) * spacing
        for _ in range(max_tries):
            x, y = vesicle_shape(N, rng, reduced_area)
            cx = cx0 + rng.uniform(-jitter, jitter)
            cy = cy0 + rng.uniform(-jitter, jitter)
            x = x + cx
            y = y + cy
            if all(_min_gap(x, y, X[:N, j], X[N:, j]) >= min_gap for j in placed):
                break
        else:
            raise RuntimeError("lattice_suspension: could not place vesicle %d" % k)
        X[:N, k] = x
        X[N:, k] = y
        placed.append(k)
    return X


def random_suspension(nv: int, N: int, area_fraction: float, min_gap: float = 0.05,
                      reduced_area=0.65, area: float = math.pi, seed: int = 0,
                      max_tries: int = 2000):
    """``nv`` vesicles with centres uniform in a square sized for the area fraction.

    ``reduced_area`` is a float or a (lo, hi) range sampled uniformly per
    vesicle.  Candidates are rejected when any point comes within
    ``min_gap`` of an already placed vesicle (cell-list search on centres).
    """
    rng = np.random.default_rng(seed)
    side = math.sqrt(nv * area / area_fraction)
    X = np.zeros((2 * N, nv))
    rmax = np.zeros(nv)
    cen = np.zeros((nv, 2))
    cell = 2.0 * ellipse_axes(min(reduced_area) if isinstance(reduced_area, tuple) else reduced_area, area)[0] * 1.2 + min_gap
    ncell = max(1, int(side // cell))
    grid: dict = {}
    for k in range(nv):
        for _ in range(max_tries):
            ra = rng.uniform(*reduced_area) if isinstance(reduced_area, tuple) else reduced_area
            x, y = vesicle_shape(N, rng, ra, area)
            cx, cy = rng.uniform(0, side, size=2)
            r = float(np.sqrt(x ** 2 + y ** 2).max())
            gx, gy = int(cx / side * ncell), int(cy / side * ncell)
            nb = [j for ix in range(gx - 1, gx + 2) for iy in range(gy - 1, gy + 2)
                  for j in grid.get((ix, iy), ())]
            ok = True
            if nb:
                nb = np.asarray(nb)
                dc = np.hypot(cx - cen[nb, 0], cy - cen[nb, 1])
                for j in nb[dc <= r + rmax[nb] + min_gap]:
                    if _min_gap(x + cx, y + cy, X[:N, j], X[N:, j]) < min_gap:
                        ok = False
                        break
            if ok:
                break
        else:
            raise RuntimeError("random_suspension: could not place vesicle %d" % k)
        X[:N, k] = x + cx
        X[N:, k] = y + cy
        rmax[k] = r
        cen[k] = (cx, cy)
        grid.setdefault((gx, gy), []).append(k)
    return X


def mixed_suspension(groups, area_fraction: float, box_aspect: float = 1.0, min_gap: float = 0.05,
                     reduced_area=0.65, area: float = math.pi, seed: int = 0, max_tries: int = 2000):
    """Vesicles of several point counts: ``groups`` = [(nv_g, N_g), ...].

    Centres uniform in a [0, Lx] x [-Ly/2, Ly/2] rectangle with Lx / Ly =
    ``box_aspect``, sized for the area fraction; vesicles are placed in a
    seeded random order over the groups with the rejection rule of
    ``random_suspension``.  Returns a list of X[2N_g, nv_g] arrays.
    """
    rng = np.random.default_rng(seed)
    nv_tot = sum(nv for nv, _ in groups)
    tot_area = nv_tot * area / area_fraction
    Ly = math.sqrt(tot_area / box_aspect)
    Lx = tot_area / Ly
    Xs = [np.zeros((2 * N, nv)) for nv, N in groups]
    order = np.concatenate([np.full(nv, g) for g, (nv, _) in enumerate(groups)])
    rng.shuffle(order)
    ra_lo = min(reduced_area) if isinstance(reduced_area, tuple) else reduced_area
    cell = 2.0 * ellipse_axes(ra_lo, area)[0] * 1.2 + min_gap
    nx, ny = max(1, int(Lx // cell)), max(1, int(Ly // cell))
    grid: dict = {}
    placed = []   # (group, column, cx, cy, r)
    count = [0] * len(groups)
    for g in order:
        N = groups[g][1]
        for _ in range(max_tries):
            ra = rng.uniform(*reduced_area) if isinstance(reduced_area, tuple) else reduced_area
            x, y = vesicle_shape(N, rng, ra, area)
            cx, cy = rng.uniform(0, Lx), rng.uniform(-0.5 * Ly, 0.5 * Ly)
            r = float(np.sqrt(x ** 2 + y ** 2).max())
            gx, gy = int(cx / Lx * nx), int((cy + 0.5 * Ly) / Ly * ny)
            ok = True
            for ix in range(gx - 1, gx + 2):
                for iy in range(gy - 1, gy + 2):
                    for q in grid.get((ix, iy), ()):
                        pg, pc, pcx, pcy, pr = placed[q]
                        if math.hypot(cx - pcx, cy - pcy) > r + pr + min_gap:
                            continue
                        Np = groups[pg][1]
                        Xp = Xs[pg]
                        if _min_gap(x + cx, y + cy, Xp[:Np, pc], Xp[Np:, pc]) < min_gap:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if ok:
                break
        else:
            raise RuntimeError("mixed_suspension: could not place a vesicle of group %d" % g)
        c = count[g]
        Xs[g][:N, c] = x + cx
        Xs[g][N:, c] = y + cy
        count[g] += 1
        grid.setdefault((gx, gy), []).append(len(placed))
        placed.append((g, c, cx, cy, r))
    return Xs


def config1_suspension(N: int = 32, seed: int = 0):
    """nv=16 vesicles of reduced area 0.65, area pi, on a 4x4 lattice, spacing 3.0, gap >= 0.3."""
    return lattice_suspension(4, N, spacing=3.0, jitter=0.1, min_gap=0.3, seed=seed)
