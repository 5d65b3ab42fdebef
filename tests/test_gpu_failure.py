"""Failure handling without a GPU fault: a bounded device-side wait that
runs out records VES_ERR_TIMEOUT in the context's status word, the call
returns that code, and the context stays usable for the next calls."""
import time

import numpy as np
import pytest
import torch

from oracle import ves2d_oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(golden):
    from ves2dpy_gb300 import _native as nat
    from ves2dpy_gb300.capsules import capsules
    dev = torch.device("cuda:0")
    ctx = nat.context(32, dev)
    t0 = time.perf_counter()
    rc = ctx.lib.ves_probe_wait_timeout(ctx.handle, nat.stream_ptr(dev))
    waited = time.perf_counter() - t0
    assert rc == nat.VES_ERR_TIMEOUT, rc
    assert "wait probe" in nat.last_error()
    assert waited < 10.0, waited
    # the same context computes correctly afterwards
    X = golden("capsules_fp64")["X32"]
    ves = capsules(torch.tensor(X, device=dev), None, None, 1.0, 1.0)
    sa, tang, cur = O.diff_prop(X)
    assert np.abs(ves.sa.cpu().numpy() - sa).max() < 1e-10 * np.abs(sa).max()
    assert np.abs(ves.cur.cpu().numpy() - cur).max() < 1e-9 * np.abs(cur).max()
    print(f"bounded wait gave up after {waited * 1e3:.0f} ms")
