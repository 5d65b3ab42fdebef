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
