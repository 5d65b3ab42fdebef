"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports exactly the entry points declared in include/ves2d_gb300.h."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "ves2d_gb300.h")).read()
    return set(re.findall(r"VES_API\s+(?:int|size_t|long long|const char\*)\s+(ves_\w+)\s*\(", txt))


def test_header_declares_api():
    names = declared()
    assert {"ves_ctx_create", "ves_biem_step", "ves_farfield", "ves_near_sing_int", "ves_stokes_sl_matrix"} <= names


def test_library_exports_every_declared_symbol():
    from ves2dpy_gb300.build import build
    lib = build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = declared() - exported
    assert not missing, missing


def test_ctypes_binds_every_symbol():
    from ves2dpy_gb300 import _native as nat
    lib = nat.load_library()
    assert set(nat.SIGNATURES) == declared()
    for name in nat.SIGNATURES:
        assert getattr(lib, name) is not None


def test_no_gpu_means_loud_failure():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from ves2dpy_gb300 import _native as nat
    with pytest.raises(ValueError):
        nat.context(32, "cpu")
