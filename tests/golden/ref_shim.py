"""Test-only import shim for the Ves2Dpy reference (``mytorch/`` variant).

This module exists only so that ``make_golden.py`` can run the reference
Python code in this development container and record its outputs as golden
fixtures.  Nothing in the product package imports it, and it is never run on
the GPU host (the reference tree is not present there).

What the shim does, and why (reference file:line in brackets):

* ``cupy`` / ``cupyx.scipy.sparse.linalg`` are imported unconditionally by
  ``mytorch/tstep_biem.py:10-14``; they are replaced by tiny stand-ins whose
  ``gmres``/``LinearOperator`` are SciPy's (the CPU branch the reference
  itself takes when CUDA is absent).
* ``torch.set_default_dtype(torch.float64)`` is restored after import, since
  ``poten.py:10``, ``filter.py:3`` and ``tstep_biem.py:4`` reset it to float32
  at import time while ``biem_support.py:2`` sets float64.
* ``promote=True`` additionally rebinds ``torch.float32``/``torch.cfloat``/
  ``torch.complex64`` and ``Tensor.float``/``Tensor.cfloat`` to their 64-bit
  counterparts before the reference modules are imported.  The reference then
  runs its own algorithm entirely in FP64 (its explicit FP32 casts, e.g.
  ``poten.py:47, 943``, ``fft1.py:76, 191, 205``, become FP64), which is what
  the FP64 parity tolerance of the GPU path is pinned against.  With
  ``promote=False`` the reference runs with its own mixed FP32/FP64 casts.
"""
import os
import sys
import types

REF_ROOT = os.environ.get("VES2D_REFERENCE", "/root/reference")


def _install_cupy_stub():
    import numpy as np
    import scipy.sparse.linalg as sla

    cp = types.ModuleType("cupy")
    cp.ndarray = type("ndarray_stub", (), {})  # never matches a real array
    cp.asarray = np.asarray
    cupyx = types.ModuleType("cupyx")
    cupyx_scipy = types.ModuleType("cupyx.scipy")
    cupyx_sparse = types.ModuleType("cupyx.scipy.sparse")
    cupyx_linalg = types.ModuleType("cupyx.scipy.sparse.linalg")
    cupyx_linalg.gmres = sla.gmres
    cupyx_linalg.LinearOperator = sla.LinearOperator
    cupyx.scipy = cupyx_scipy
    cupyx_scipy.sparse = cupyx_sparse
    cupyx_sparse.linalg = cupyx_linalg
    sys.modules.setdefault("cupy", cp)
    sys.modules.setdefault("cupyx", cupyx)
    sys.modules.setdefault("cupyx.scipy", cupyx_scipy)
    sys.modules.setdefault("cupyx.scipy.sparse", cupyx_sparse)
    sys.modules.setdefault("cupyx.scipy.sparse.linalg", cupyx_linalg)


def _promote_torch_to_fp64():
    import torch

    torch.float32 = torch.float64
    torch.float = torch.float64
    torch.cfloat = torch.cdouble
    torch.complex64 = torch.complex128
    torch.Tensor.float = torch.Tensor.double
    torch.Tensor.cfloat = torch.Tensor.cdouble
    _set = torch.set_default_dtype

    def _always64(_dtype):
        _set(torch.float64)

    torch.set_default_dtype = _always64


def load(promote: bool = True, variant: str = "mytorch"):
    """Import the reference modules and return them in a namespace."""
    import torch

    torch.set_default_device("cpu")
    _install_cupy_stub()
    if promote:
        _promote_torch_to_fp64()
    path = os.path.join(REF_ROOT, variant)
    if path not in sys.path:
        sys.path.insert(0, path)
    import fft1
    import filter as ref_filter
    import curve_batch_compile
    import capsules
    import biem_support
    import poten
    import tstep_biem

    torch.set_default_dtype(torch.float64)
    torch.set_default_device("cpu")
    ns = types.SimpleNamespace(
        fft1=fft1, filter=ref_filter, curve=curve_batch_compile,
        capsules=capsules, biem_support=biem_support, poten=poten,
        tstep_biem=tstep_biem, torch=torch,
    )
    return ns


def load_mlarm(precision: str = "fp64"):
    """Import the reference MLARM N=128 wrapper (``newtorch/``) for golden runs.

    Import order follows the reference driver
    (``newtorch/entry_driver_manyfreeSpaceVesicle_N128.py:1-20``): the
    ``newtorch`` modules come first, ``newtorch/tools`` provides ``filter``,
    the project root provides ``model_zoo``, and ``fft1`` (absent from
    ``newtorch``) comes from ``mytorch``.  ``torch.compile`` is replaced by
    the identity, so the ``@torch.compile(backend='cudagraphs')`` methods
    (``wrapper_MLARM_batch_compile_N128.py:4140,4154``) run eagerly on CPU.

    As written, the reference step cannot run with stock PyTorch in either
    dtype: with float64 shapes ``redistributeArcLength`` writes a complex64
    result into the float64 ``X`` (``curve_batch_compile.py:962-970``,
    "Index put requires the source and destination dtypes match"), and with
    float32 shapes ``buildVelocityInNear`` multiplies ``.double()`` network
    outputs with a float32 force (``wrapper_MLARM_batch_compile_N128.py:1831``,
    "expected scalar type Float but found Double").  Two minimal patches make
    it run:

    * ``precision="mixed"``: ``Tensor.cfloat`` returns complex128, so the
      geometry runs in FP64 and the networks in the reference's FP32
      (``.float()`` casts in ``model_zoo/get_network_torch.py``) -- the
      combination the driver sets up (float64 initial shapes,
      ``entry_driver_manyfreeSpaceVesicle_N128.py:4,100``);
    * ``precision="fp64"``: the whole reference, networks included (the
      caller converts the loaded models with ``.double()``), runs in FP64
      through the same rebinding ``load(promote=True)`` uses.
    """
    import torch

    torch.set_default_device("cpu")
    _install_cupy_stub()
    if precision == "fp64":
        _promote_torch_to_fp64()
    elif precision == "mixed":
        torch.Tensor.cfloat = torch.Tensor.cdouble
    else:
        raise ValueError(precision)

    def _identity_compile(fn=None, **_kw):
        if fn is None:
            return lambda f: f
        return fn

    torch.compile = _identity_compile
    # model_zoo/Net_ves_factor.py:3 and Net_ves_merge_nocoords_nearFourier.py:3
    # import torchsummary (a printing helper they never call).
    ts = types.ModuleType("torchsummary")
    ts.summary = lambda *a, **k: None
    sys.modules.setdefault("torchsummary", ts)
    for sub in ("mytorch", "", "newtorch/tools", "newtorch"):
        p = os.path.join(REF_ROOT, sub) if sub else REF_ROOT
        if p in sys.path:
            sys.path.remove(p)
        sys.path.insert(0, p)
    import wrapper_MLARM_batch_compile_N128 as wrapper
    import curve_batch_compile
    import capsules
    import biem_support
    import filter as ref_filter
    import poten
    from model_zoo import (Net_ves_factor, Net_ves_merge_adv, Net_ves_selften,
                           Net_ves_merge_advten, Net_ves_merge_nocoords_nearFourier)

    ns = types.SimpleNamespace(
        wrapper=wrapper, curve=curve_batch_compile, capsules=capsules,
        biem_support=biem_support, filter=ref_filter, poten=poten, torch=torch,
        nets=types.SimpleNamespace(
            relax=Net_ves_factor.pdeNet_Ves_factor_periodic,
            adv=Net_ves_merge_adv.Net_merge_advection,
            selften=Net_ves_selften.Net_ves_selften,
            advten=Net_ves_merge_advten.Net_ves_merge_advten,
            near=Net_ves_merge_nocoords_nearFourier.Net_ves_merge_nocoords_nearFourier,
        ),
    )
    return ns
