"""GPU tests of the multipole all-pairs path (precision "fp32m").

The reference sums every (target point, upsampled source point) pair
(biem_support.py:7-272, poten.py:280-336).  "fp32m" evaluates separated
vesicle pairs through a truncated multipole expansion of the source vesicle
(truncation bound 1e-10 of the source's density magnitude) and the others by
the direct FP32 rule, so it is checked against the FP64 direct sum: random
suspensions where most pairs are separated, the golden far-field cases with
near-pair exclusions, and MLARM steps.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
UNIT_AREA = 0.65 / (4 * math.pi)   # reduced area 0.65 at unit length
FP32_TOL = 1e-5                    # the FP32 far-field tolerance of the suite


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _suspension(nv, N, ns, frac, seed):
    """Sources: nv closed curves of ns points; targets: every (ns/N)-th point;
    densities: smooth, force-free, quadrature-weighted."""
    from ves2dpy_gb300.suspension import random_suspension
    X = random_suspension(nv, ns, frac, min_gap=0.01, area=UNIT_AREA, seed=seed)   # [2 ns, nv]
    step = ns // N
    Xt = np.concatenate([X[:ns:step], X[ns::step]], axis=0)                        # [2 N, nv]
    rng = np.random.default_rng(seed + 1)
    th = 2 * np.pi * np.arange(ns) / ns
    den = np.zeros((nv, 2 * ns))
    for v in range(nv):
        for c in range(2):
            a = rng.normal(size=8) / np.arange(1, 9) ** 2
            b = rng.normal(size=8) / np.arange(1, 9) ** 2
            fc = sum(a[k] * np.cos((k + 1) * th) + b[k] * np.sin((k + 1) * th) for k in range(8))
            den[v, c * ns:(c + 1) * ns] = fc * (2 * np.pi / ns)
    to = lambda A: torch.from_numpy(np.ascontiguousarray(A)).to(DEV)
    return to(X.T), to(den), to(Xt.T)


@pytest.mark.parametrize("N,ns,nv,frac", [(128, 1536, 256, 0.15), (32, 192, 600, 0.30)])
def test_multipole_matches_direct_sum(N, ns, nv, frac):
    from ves2dpy_gb300.biem_support import _farfield
    Xs, den, Xt = _suspension(nv, N, ns, frac, seed=5)
    self_idx = torch.arange(nv, dtype=torch.int32, device=DEV)
    ref = _farfield("fp64", Xs, den, Xt, self_idx, None, N)
    got = _farfield("fp32m", Xs, den, Xt, self_idx, None, N)
    c32 = _farfield("fp32c", Xs, den, Xt, self_idx, None, N)
    err, err_c = rel(got, ref), rel(c32, ref)
    # the FP32 series lose no more than the FP32C direct rule (a few 1e-8 here)
    assert err < 1e-6 and err < 20 * max(err_c, 1e-9), (err, err_c)


def test_multipole_without_self_exclusion():
    """Targets that are not on any source vesicle, no self index."""
    from ves2dpy_gb300.biem_support import _farfield
    Xs, den, Xt = _suspension(128, 32, 192, 0.15, seed=9)
    Xt = Xt + 0.37   # shifted copies of the curves: mostly between the sources
    ref = _farfield("fp64", Xs, den, Xt, None, None, 32)
    got = _farfield("fp32m", Xs, den, Xt, None, None, 32)
    assert rel(got, ref) < 1e-6


def test_far_field_compare_multipole(golden):
    """The golden far-field cases (near-pair exclusions from the reference's
    near-zone lists)."""
    from ves2dpy_gb300 import biem_support as B
    T = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64, device=DEV)
    g = golden("far_fp64")
    far2 = B.allExactStokesSLTarget_compare2(T(g["Xup"]), T(g["sa_up"]), T(g["fup"]), T(g["X"]), g["ids0"],
                                             g["ids1"], g["ids2"], precision="fp32m")
    assert rel(far2, g["far2"]) < FP32_TOL
    far1, ids = B.allExactStokesSLTarget_compare1(T(g["Xup"]), T(g["sa_up"]), T(g["fup"]), T(g["X"]),
                                                  precision="fp32m")
    assert rel(far1, g["far1"]) < FP32_TOL
    for got, key in zip(ids, ["c1_ids0", "c1_ids1", "c1_ids2"]):
        np.testing.assert_array_equal(got, g[key])
