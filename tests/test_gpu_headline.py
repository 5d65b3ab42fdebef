"""The headline suspension through 25 consecutive MLARM steps (the bench's
warm-up and timed steps): 4096 unit-length vesicles of N=128 at 15% area
fraction in shear flow of rate 2, dt=1e-5, prepared as the reference driver
prepares its initial shapes (entry_driver_manyfreeSpaceVesicle_N128.py:157-167),
with the trained networks.  The near lists are sized on the device and grown
by the caller, so no step may overflow them; the shapes stay finite and
their areas and lengths within the step's correction tolerance."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
UNIT_AREA = 0.65 / (4 * math.pi)  # reduced area 0.65 at unit length
MIN_GAP = 0.05 / 7.79             # the 0.05 gap of radius-1 vesicles at unit length


def test_headline_suspension_runs_25_steps():
    from ves2dpy_gb300 import training as TR
    from ves2dpy_gb300.curve import Curve
    from ves2dpy_gb300.mlarm import MLARM_manyfree_py
    from ves2dpy_gb300.mlarm_weights import NETS, synthetic_norms, synthetic_state_dict
    from ves2dpy_gb300.suspension import random_suspension

    if TR.have_trained():
        sds, norms = TR.load()
    else:
        sds, norms = {n: synthetic_state_dict(n, 0) for n in NETS}, synthetic_norms(0)
    nrm = {k: torch.from_numpy(np.asarray(v, dtype=np.float64)) for k, v in norms.items()}

    def vinf(X):
        n = X.shape[0] // 2
        return 2.0 * torch.vstack((X[n:], torch.zeros_like(X[:n])))

    m = MLARM_manyfree_py(1e-5, vinf, Curve(), False, 1e2, -1, nrm["adv_in"], nrm["adv_out"], nrm["relax_in"],
                          nrm["relax_out"], nrm["near_in"], nrm["near_out"], nrm["selften_in"], nrm["selften_out"],
                          nrm["advten_in"], nrm["advten_out"], DEV, state_dicts=sds, net_precision="bf16",
                          farfield_precision="fp32m")
    X = torch.tensor(random_suspension(4096, 128, 0.15, min_gap=MIN_GAP, area=UNIT_AREA, seed=0),
                     dtype=torch.float64, device=DEV)
    cv = Curve()
    _, area0, len0 = cv.geomProp(X)
    for _ in range(10):
        X, good = cv.redistributeArcLength(X)
        if good:
            break
    m.area0, m.len0 = area0, len0
    ten = torch.zeros(128, 4096, dtype=torch.float64, device=DEV)
    for _ in range(25):
        X, ten = m.time_step_many_noinfo(X, ten, 3)
    assert torch.isfinite(X).all() and torch.isfinite(ten).all()
    _, a1, l1 = cv.geomProp(X)
    drift = max(float(((a1 - area0).abs() / area0).max()), float(((l1 - len0).abs() / len0).max()))
    assert drift < 2e-2, drift
    assert m.last_result.n_near_pairs > 0
