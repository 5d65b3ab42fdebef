"""Trajectory writer with device frames and the device ``Curve.ellipse``
against the reference (golden io_fp64)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def test_ellipse_on_device_matches_reference(golden):
    from ves2dpy_gb300.curve import Curve
    g = golden("io_fp64")
    oc = Curve()
    for N, ra in ((32, 0.65), (64, 0.9), (128, 0.5), (16, 0.75)):
        ref = g[f"ellipse_{N}_{int(round(ra * 100))}"]
        got = oc.ellipse(N, torch.tensor([ra], dtype=torch.float64)).cpu().numpy()
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max(), (N, ra)


def test_writer_device_frames_bytes(golden, tmp_path):
    from ves2dpy_gb300.trajectory import TrajectoryWriter
    g = golden("io_fp64")
    p = tmp_path / "d.bin"
    with TrajectoryWriter(p, torch.from_numpy(g["traj_X0"]).to(DEV)) as w:
        for t, X in zip(g["traj_times"], g["traj_frames"]):
            w.append(float(t), torch.from_numpy(X).to(DEV))
    assert np.array_equal(np.fromfile(p, dtype=np.uint8), g["traj_bytes"])


def test_writer_copies_in_stream_order(tmp_path):
    """A frame holds the values the array had when it was appended, although
    the array is overwritten right after on the same stream."""
    from ves2dpy_gb300.trajectory import TrajectoryWriter, load_ves2d_file
    N, nv, nframes = 128, 256, 12
    X = torch.zeros(2 * N, nv, dtype=torch.float64, device=DEV)
    p = tmp_path / "s.bin"
    with TrajectoryWriter(p, X, nslots=3) as w:
        for k in range(nframes):
            X.fill_(float(k + 1))
            w.append(1e-5 * (k + 1), X)
            X.mul_(-7.0)   # queued after the copy: must not reach the file
    vx, vy, t, *_ = load_ves2d_file(p)
    assert vx.shape == (N, nv, nframes)
    for k in range(nframes):
        assert np.all(vx[:, :, k] == k + 1) and np.all(vy[:, :, k] == k + 1)
    assert np.allclose(t, 1e-5 * np.arange(1, nframes + 1), rtol=0, atol=0)


def test_repulsion_force_matches_reference(golden):
    """Device repulsion (bounding-box candidates, exact pair sums) vs the
    reference's dense evaluation."""
    from ves2dpy_gb300.capsules import capsules
    g = golden("repulsion_fp64")
    for tag in ("tight", "wide"):
        X = torch.from_numpy(g[f"X_{tag}"]).to(DEV)
        ves = capsules(X, None, None, 1.0, 1.0)
        got = ves.repulsionForce(X, float(g[f"W_{tag}"]), float(g[f"eta_{tag}"])).cpu().numpy()
        ref = g[f"rep_{tag}"]
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max(), tag


def test_repulsion_force_large_suspension():
    """nv=2048 random suspension against the oracle on a subset of target
    vesicles (all sources)."""
    from oracle import ves2d_oracle as O
    from ves2dpy_gb300.capsules import capsules
    from ves2dpy_gb300.suspension import random_suspension
    N, nv, eta, W = 32, 2048, 0.05, 900.0
    X = random_suspension(nv, N, 0.30, min_gap=0.01, area=0.65 / (4 * np.pi), seed=4)
    Xd = torch.from_numpy(X).to(DEV)
    got = capsules(Xd, None, None, 1.0, 1.0).repulsionForce(Xd, W, eta).cpu().numpy()
    ref_all = np.zeros_like(X)
    cols = np.arange(0, nv, 97)
    for a in cols:
        # the dense restatement on the target vesicle plus its neighbours within reach
        c = X.reshape(2, N, nv).mean(axis=1)
        near = np.where(np.hypot(c[0] - c[0, a], c[1] - c[1, a]) < 1.0)[0]
        sub = X[:, near]
        r = O.repulsion_force(sub, W, eta)
        ref_all[:, a] = r[:, list(near).index(a)]
    ref = ref_all[:, cols]
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.abs(ref).max() > 0
    assert np.abs(got[:, cols] - ref).max() < 1e-11 * scale
