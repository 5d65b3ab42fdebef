"""GB300-native (sm_103a) implementation of the Ves2Dpy boundary-integral
vesicle-suspension step.

The public classes keep the reference's names and call signatures:
``Poten`` (poten.py), ``capsules`` (capsules.py), ``Curve``
(curve_batch_compile.py), ``TStepBiem`` (tstep_biem.py) and the
``biem_support`` / ``filter`` functions.  They operate on CUDA tensors and call
the C-ABI library ``_lib/libves2d_gb300.so`` (declared in
``include/ves2d_gb300.h``); there is no CPU fallback.
"""
from ._native import GmresNotConverged, NearListOverflow, VesError, load_library  # noqa: F401
from .suspension import config1_suspension, lattice_suspension, mixed_suspension, random_suspension  # noqa: F401

__all__ = ["Poten", "capsules", "Curve", "TStepBiem", "TStepBiemMixed", "naiveNearZoneInfo", "load_library",
           "config1_suspension", "lattice_suspension", "mixed_suspension", "random_suspension"]


def __getattr__(name):
    if name == "Poten":
        from .poten import Poten
        return Poten
    if name == "capsules":
        from .capsules import capsules
        return capsules
    if name == "Curve":
        from .curve import Curve
        return Curve
    if name == "TStepBiem":
        from .tstep_biem import TStepBiem
        return TStepBiem
    if name == "TStepBiemMixed":
        from .tstep_biem import TStepBiemMixed
        return TStepBiemMixed
    if name == "naiveNearZoneInfo":
        from .biem_support import naiveNearZoneInfo
        return naiveNearZoneInfo
    raise AttributeError(name)
