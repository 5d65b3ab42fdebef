"""The all-pairs sum through ``ves_farfield_static_scratch``.

That entry point serves callers that cannot allocate device memory when they
call (an application whose GPU memory is entirely owned by its own pool, or a
host calling in from a runtime where cudaMalloc would synchronise the device):
its scratch is a fixed array inside the library image instead of a workspace
the caller allocates.  The test calls it through the C ABI twice in a row and
checks both results against the workspace-based ``ves_farfield`` at the same
tolerances as the other parity tests, for FP64, FP32C and FP32M (the
multipole path), checks that the second call changes neither the device's
free memory nor the caching allocator's reservation, and checks that a size
whose scratch does not fit is rejected.  The file name makes pytest collect
it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32c": 1e-5, "fp32m": 1e-5}


def _inputs(dev):
    from ves2dpy_gb300.suspension import lattice_suspension
    X = lattice_suspension(3, 32, spacing=3.0, jitter=0.1, min_gap=0.3, seed=4)  # 9 vesicles, N=32
    N, nv = X.shape[0] // 2, X.shape[1]
    rng = np.random.default_rng(5)
    den = rng.normal(size=X.shape) * 1e-2
    Xv = torch.tensor(X.T.copy(), dtype=torch.float64, device=dev)      # [nv][2][N]
    dv = torch.tensor(den.T.copy(), dtype=torch.float64, device=dev)
    self_idx = torch.arange(nv, dtype=torch.int32, device=dev)
    return Xv, dv, self_idx, N, nv


@pytest.mark.parametrize("precision", ["fp64", "fp32c", "fp32m"])
def test_static_scratch_matches_workspace_entry_twice(precision):
    from ves2dpy_gb300 import _native as nat
    dev = torch.device("cuda:0")
    lib = nat.load_library()
    Xv, dv, self_idx, N, nv = _inputs(dev)
    prec = nat.PREC[precision]
    stream = nat.stream_ptr(dev)

    ctx = nat.context(N, dev)
    ref = torch.empty(nv, 2 * N, dtype=torch.float64, device=dev)
    ws = torch.empty(lib.ves_farfield_workspace(ctx.handle, prec, nv, N, nv, N), dtype=torch.uint8, device=dev)
    nat.check(lib.ves_farfield(ctx.handle, prec, nv, N, Xv.data_ptr(), dv.data_ptr(), nv, N, Xv.data_ptr(),
                               self_idx.data_ptr(), None, ref.data_ptr(), ws.data_ptr(), ws.numel(), stream))
    refn = ref.cpu().numpy()
    scale = np.abs(refn).max()
    assert scale > 0
    outs = [torch.full((nv, 2 * N), float("nan"), dtype=torch.float64, device=dev) for _ in range(2)]
    for call in range(2):
        torch.cuda.synchronize(dev)
        free0, reserved0 = torch.cuda.mem_get_info(dev)[0], torch.cuda.memory_reserved(dev)
        rc = lib.ves_farfield_static_scratch(prec, nv, N, Xv.data_ptr(), dv.data_ptr(), nv, N, Xv.data_ptr(),
                                             self_idx.data_ptr(), outs[call].data_ptr(), stream)
        nat.check(rc, f"static scratch call {call}")
        torch.cuda.synchronize(dev)
        if call == 1:  # the first call may load the kernels; the second allocates nothing
            assert torch.cuda.mem_get_info(dev)[0] == free0
            assert torch.cuda.memory_reserved(dev) == reserved0
        err = np.abs(outs[call].cpu().numpy() - refn).max() / scale
        assert err < TOL[precision], (precision, call, err)


def test_static_scratch_rejects_oversized():
    from ves2dpy_gb300 import _native as nat
    dev = torch.device("cuda:0")
    lib = nat.load_library()
    nsrc, ns, ntp = 4096, 1536, 128  # source records alone: 4096*1536*16 B = 96 MiB > 64 MiB
    Xs = torch.zeros(nsrc, 2 * ns, dtype=torch.float64, device=dev)
    ds = torch.zeros_like(Xs)
    Xt = torch.zeros(1, 2 * ntp, dtype=torch.float64, device=dev)
    out = torch.zeros_like(Xt)
    rc = lib.ves_farfield_static_scratch(nat.PREC["fp32c"], nsrc, ns, Xs.data_ptr(), ds.data_ptr(), 1, ntp,
                                         Xt.data_ptr(), None, out.data_ptr(), nat.stream_ptr(dev))
    assert rc == nat.VES_ERR_WORKSPACE
    assert "static array holds" in nat.last_error()
