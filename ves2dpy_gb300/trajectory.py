"""Trajectory files in the reference's binary format.

The drivers write (mytorch/driver_confined.py:204-206, 294-296)

    [N, nv] + X.T.flatten()           once, the initial shapes
    [time] + X.T.flatten()            once per step

as little-endian float64, with X the reference's [2N, nv] array (N x rows
then N y rows per vesicle), and newtorch/tools/load_ves2d_file.py:4-72 reads
them back.  ``TrajectoryWriter`` writes the same bytes through the C library:
device frames are copied asynchronously into pinned buffers on the current
stream and a background thread writes them, so the step never waits for the
disk.  ``load_ves2d_file`` returns what the reference's reader returns.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as nat
from .layout import from_vm, to_vm


def _device_frame(X: torch.Tensor) -> torch.Tensor:
    """[2N, nv] (reference layout) -> contiguous [nv][2][N] (the file's frame order)."""
    return to_vm(X) if X.dim() == 2 else X.reshape(1, -1).to(torch.float64).contiguous()


class TrajectoryWriter:
    """``TrajectoryWriter(fileName, X0)`` creates the file with the header and
    the initial shapes X0 [2N, nv]; ``append(time, X)`` adds one frame;
    ``close()`` (or leaving a ``with`` block) waits for the last frame."""

    def __init__(self, fileName: str, X0: torch.Tensor, nslots: int = 3):
        self.lib = nat.load_library()
        N, nv = X0.shape[0] // 2, (X0.shape[1] if X0.dim() == 2 else 1)
        self.N, self.nv = N, nv
        self.nslots = max(1, nslots)
        F = _device_frame(X0)
        self._hold = []
        h = ctypes.c_void_p()
        on_dev = 1 if F.is_cuda else 0
        nat.check(self.lib.ves_traj_create(str(fileName).encode(), N, nv, F.data_ptr(), on_dev, nslots,
                                           ctypes.byref(h)), "trajectory create")
        self.handle = h

    def append(self, time: float, X: torch.Tensor) -> None:
        if self.handle is None:
            raise ValueError("trajectory is closed")
        if X.shape[0] // 2 != self.N or (X.shape[1] if X.dim() == 2 else 1) != self.nv:
            raise ValueError("frame shape %s does not match N=%d, nv=%d" % (tuple(X.shape), self.N, self.nv))
        F = _device_frame(X)
        # the asynchronous copy reads F in stream order; keep the last frames
        # referenced until they are written (more than the slots in flight)
        self._hold.append(F)
        if len(self._hold) > self.nslots + 1:
            self._hold.pop(0)
        stream = nat.stream_ptr(F.device) if F.is_cuda else None
        nat.check(self.lib.ves_traj_append(self.handle, float(time), F.data_ptr(), 1 if F.is_cuda else 0, stream),
                  "trajectory append")

    def flush(self) -> int:
        n = ctypes.c_longlong(0)
        nat.check(self.lib.ves_traj_flush(self.handle, ctypes.byref(n)), "trajectory flush")
        self._hold.clear()
        return int(n.value)

    def close(self) -> None:
        if self.handle is not None:
            rc = self.lib.ves_traj_close(self.handle)
            self.handle = None
            self._hold.clear()
            nat.check(rc, "trajectory close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_ves2d_file(filename):
    """Read a trajectory file: returns ``(vesx, vesy, time, N, nv, xinit, yinit)``
    with vesx, vesy of shape (N, nv, ntime), as
    newtorch/tools/load_ves2d_file.py:4-72 (vectorised; a trailing partial
    frame is ignored, as there)."""
    val = np.fromfile(filename, dtype=np.float64)
    N, nv = int(val[0]), int(val[1])
    n_init = 2 * N * nv
    init = val[2:2 + n_init].reshape(nv, 2, N)
    xinit = np.ascontiguousarray(init[:, 0, :].T)
    yinit = np.ascontiguousarray(init[:, 1, :].T)
    rest = val[2 + n_init:]
    stride = n_init + 1
    ntime = rest.size // stride
    frames = rest[:ntime * stride].reshape(ntime, stride)
    time = frames[:, 0].copy()
    shp = frames[:, 1:].reshape(ntime, nv, 2, N)
    vesx = np.ascontiguousarray(shp[:, :, 0, :].transpose(2, 1, 0))
    vesy = np.ascontiguousarray(shp[:, :, 1, :].transpose(2, 1, 0))
    return vesx, vesy, time, N, nv, xinit, yinit
