"""Trajectory files and geometry tooling (CPU): the oracle pinned to the
reference's own reader and ellipse (golden io_fp64), the C-ABI writer with
host frames, the vectorised reader and the driver defaults."""
import os

import numpy as np
import pytest

from oracle import ves2d_oracle as O


def test_oracle_ellipse_matches_reference(golden):
    g = golden("io_fp64")
    for N, ra in ((32, 0.65), (64, 0.9), (128, 0.5), (16, 0.75)):
        ref = g[f"ellipse_{N}_{int(round(ra * 100))}"]
        got = O.ellipse(N, ra)
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max(), (N, ra)


def test_oracle_trajectory_matches_reference(golden, tmp_path):
    g = golden("io_fp64")
    p = tmp_path / "t.bin"
    O.write_trajectory(p, g["traj_X0"], list(zip(g["traj_times"], g["traj_frames"])))
    assert np.array_equal(np.fromfile(p, dtype=np.uint8), g["traj_bytes"])
    vx, vy, t, N, nv, xi, yi = O.load_ves2d_file(p)
    for got, key in ((vx, "load_vesx"), (vy, "load_vesy"), (t, "load_time"), (xi, "load_xinit"), (yi, "load_yinit")):
        assert np.array_equal(got, g[key]), key
    assert (N, nv) == (int(g["load_N"]), int(g["load_nv"]))


def test_writer_host_frames_bytes(golden, tmp_path):
    """The C-ABI writer (host frames, no GPU needed) writes the reference's bytes."""
    torch = pytest.importorskip("torch")
    from ves2dpy_gb300.trajectory import TrajectoryWriter
    g = golden("io_fp64")
    p = tmp_path / "w.bin"
    with TrajectoryWriter(p, torch.from_numpy(g["traj_X0"]), nslots=2) as w:
        for t, X in zip(g["traj_times"], g["traj_frames"]):
            w.append(float(t), torch.from_numpy(X))
        assert w.flush() == len(g["traj_times"])
    assert np.array_equal(np.fromfile(p, dtype=np.uint8), g["traj_bytes"])


def test_reader_matches_reference_reader(golden, tmp_path):
    from ves2dpy_gb300.trajectory import load_ves2d_file
    g = golden("io_fp64")
    p = tmp_path / "r.bin"
    g["traj_bytes"].tofile(p)
    got = load_ves2d_file(p)
    keys = ("load_vesx", "load_vesy", "load_time", "load_N", "load_nv", "load_xinit", "load_yinit")
    for a, key in zip(got, keys):
        assert np.array_equal(np.asarray(a), g[key]), key
    # a partly written last frame is ignored, as by the reference reader
    with open(p, "ab") as f:
        np.arange(5, dtype=np.float64).tofile(f)
    vx = load_ves2d_file(p)[0]
    assert vx.shape == g["load_vesx"].shape and np.array_equal(vx, g["load_vesx"])


def test_writer_reports_unwritable_path(tmp_path):
    torch = pytest.importorskip("torch")
    from ves2dpy_gb300.trajectory import TrajectoryWriter
    with pytest.raises(ValueError):
        TrajectoryWriter(os.path.join(tmp_path, "missing", "dir", "t.bin"), torch.zeros(8, 2, dtype=torch.float64))


def test_init_ves2d_defaults():
    """driver_confined.py:14-77: defaults fill in, unconfined runs have no
    walls, a scalar viscosity contrast becomes one entry per vesicle."""
    from ves2dpy_gb300.options import initVes2D
    options, prams = initVes2D({"farField": "vortex"}, {"nv": 3, "Nbd": 32, "viscCont": 2.0, "dt": 1e-4})
    assert options["farField"] == "vortex" and options["usePreco"] is True and options["confined"] is False
    assert prams["dt"] == 1e-4 and prams["kappa"] == 1e-1 and prams["gmresTol"] == 1e-5
    assert prams["Nbd"] == 0 and prams["nvbd"] == 0
    assert prams["viscCont"] == [2.0, 2.0, 2.0]
    options, prams = initVes2D({"confined": True}, {"Nbd": 32, "nvbd": 2})
    assert prams["Nbd"] == 32 and prams["nvbd"] == 2 and prams["viscCont"] == [1]


def test_oracle_repulsion_matches_reference(golden):
    """capsules.repulsionForce (capsules.py:209-252) restated."""
    g = golden("repulsion_fp64")
    for tag in ("tight", "wide"):
        ref = g[f"rep_{tag}"]
        got = O.repulsion_force(g[f"X_{tag}"], float(g[f"W_{tag}"]), float(g[f"eta_{tag}"]))
        assert np.abs(ref).max() > 0
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max(), tag


def test_oracle_rbf_near_field_matches_reference(golden):
    """nearSingInt_rbf (poten.py:643-894) restated: layer velocities, Gaussian
    fits (LU instead of the reference's Cholesky) and the near-pair
    correction."""
    g = golden("rbf_fp64")
    for tag in ("n32", "n128"):
        ref = g[f"LP_{tag}"]
        got = O.near_sing_int_rbf(g[f"X_{tag}"], g[f"f_{tag}"], g[f"vself_{tag}"], g[f"far_{tag}"],
                                  g[f"id1_{tag}"], g[f"id2_{tag}"])
        assert len(g[f"id1_{tag}"]) > 0
        assert np.abs(got - ref).max() < 1e-10 * np.abs(ref).max(), tag
