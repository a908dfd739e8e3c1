"""GB300-native Wilson Dslash: a drop-in for JeffersonLab/sse_wilson_dslash.

Native libraries (built in-tree by ``_build.build()``):
  lib/libgbdslash.so    sm_103a kernels + extended C ABI (include/gbdslash.h)
  lib/libgbdslash32.so  the reference's entry points, float
  lib/libgbdslash64.so  the reference's entry points, double

Python layers (thin; no compute in Python):
  legacy    mirror of the reference's C API on host arrays
  device    device-resident operator on torch CUDA tensors
  layouts   the QDP++ site orders
"""
from . import layouts  # noqa: F401

__version__ = "0.1.0"


def build(verbose: bool = False):
    from . import _build
    return _build.build(verbose=verbose)
