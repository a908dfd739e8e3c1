"""Python mirror of the reference's C API (include/sse_dslash.h,
include/sse_dslash_3d.h), on the drop-in libraries.

Same names, argument meaning and behaviour as the C functions; the arrays are
host numpy arrays in the reference's packed layouts:

    u   float[V][4][3][3][2]  (u[s][mu][j][i] = U_mu(s)_ij)
    psi float[V][4][3][2], res likewise, in the caller's site order.

``SSEDslash(32)`` binds libgbdslash32.so (float), ``SSEDslash(64)`` binds
libgbdslash64.so (double).  The module-level functions use the FP32 library,
like a C program built with SSE_PRECISION=32.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _as_callback(f, proto):
    if f is None:
        return None, None
    if isinstance(f, int):
        return f, None  # a C function address
    cb = proto(f)
    return ctypes.cast(cb, ctypes.c_void_p).value, cb


class SSEDslash:
    """The reference API for one precision (one drop-in library)."""

    def __init__(self, prec: int = 32):
        if prec not in (32, 64):
            raise ValueError("prec must be 32 or 64")
        self.prec = prec
        self.dtype = np.float32 if prec == 32 else np.float64
        self._L = _lib.legacy(prec)
        self._keep = {}

    # -- init / free ---------------------------------------------------------
    def _init(self, name, latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber):
        dims = (ctypes.c_int * 4)(*[int(v) for v in latt_size])
        gc, k1 = _as_callback(getSiteCoords, _lib.GETCOORDS)
        gl, k2 = _as_callback(getLinearSiteIndex, _lib.GETLINEAR)
        nn, k3 = _as_callback(nodeNumber, _lib.NODENUM)
        getattr(self._L, name)(dims, gc, gl, nn)
        # Python callbacks are only used during init, but keep them alive anyway.
        self._keep[name] = (k1, k2, k3)

    def init_sse_su3dslash(self, latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber=None):
        self._init("init_sse_su3dslash", latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber)

    def init_sse_su3dslash_3d(self, latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber=None):
        self._init("init_sse_su3dslash_3d", latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber)

    def free_sse_su3dslash(self):
        self._L.free_sse_su3dslash()

    def free_sse_su3dslash_3d(self):
        self._L.free_sse_su3dslash_3d()

    def sse_su3dslash_prepost_receives(self):
        self._L.sse_su3dslash_prepost_receives()

    # -- apply -----------------------------------------------------------------
    def _ptr(self, a):
        if isinstance(a, np.ndarray):
            if a.dtype != self.dtype or not a.flags["C_CONTIGUOUS"]:
                raise TypeError(f"expected a C-contiguous {np.dtype(self.dtype).name} array")
            return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float if self.prec == 32 else ctypes.c_double))
        if hasattr(a, "data_ptr"):  # a CPU torch tensor (pinned or not)
            if a.is_cuda:
                raise TypeError("the reference API takes host arrays")
            return ctypes.cast(a.data_ptr(), ctypes.POINTER(ctypes.c_float if self.prec == 32 else ctypes.c_double))
        raise TypeError("expected a numpy array or a CPU tensor")

    def sse_su3dslash_wilson(self, u, psi, res, isign, cb):
        self._L.sse_su3dslash_wilson(self._ptr(u), self._ptr(psi), self._ptr(res), int(isign), int(cb))

    def sse_su3dslash_wilson_3d(self, u, psi, res, isign, cb):
        self._L.sse_su3dslash_wilson_3d(self._ptr(u), self._ptr(psi), self._ptr(res), int(isign), int(cb))

    def pack_gauge_field(self, volume, u, u_tmp):
        self._L.pack_gauge_field(int(volume), self._ptr(u), self._ptr(u_tmp))

    def unpack_gauge_field(self, volume, u_tmp, u):
        self._L.unpack_gauge_field(int(volume), self._ptr(u_tmp), self._ptr(u))


# Legacy-path switches (extended API).
def set_exit_on_error(on: bool) -> None:
    _lib.core().gbds_legacy_set_exit_on_error(1 if on else 0)


def set_gauge_cache(on: bool) -> None:
    _lib.core().gbds_legacy_set_gauge_cache(1 if on else 0)


def invalidate_gauge() -> None:
    _lib.core().gbds_legacy_invalidate_gauge()


def set_recon(recon: int) -> None:
    _lib.check(_lib.core().gbds_legacy_set_recon(int(recon)))


def set_host_access(mode: int) -> None:
    """0: kernels read/write the caller's host arrays directly where possible; 1: stage copies."""
    _lib.check(_lib.core().gbds_legacy_set_host_access(int(mode)))


def last_path() -> int:
    """1 if the last apply used direct host access, 0 if it staged copies."""
    return int(_lib.core().gbds_legacy_last_path())


def refcount(prec: int, nd: int) -> int:
    return int(_lib.core().gbds_legacy_refcount(prec, nd))


_default = None


def _d():
    global _default
    if _default is None:
        _default = SSEDslash(32)
    return _default


def init_sse_su3dslash(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber=None):
    _d().init_sse_su3dslash(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber)


def free_sse_su3dslash():
    _d().free_sse_su3dslash()


def sse_su3dslash_wilson(u, psi, res, isign, cb):
    _d().sse_su3dslash_wilson(u, psi, res, isign, cb)


def sse_su3dslash_prepost_receives():
    _d().sse_su3dslash_prepost_receives()


def init_sse_su3dslash_3d(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber=None):
    _d().init_sse_su3dslash_3d(latt_size, getSiteCoords, getLinearSiteIndex, nodeNumber)


def free_sse_su3dslash_3d():
    _d().free_sse_su3dslash_3d()


def sse_su3dslash_wilson_3d(u, psi, res, isign, cb):
    _d().sse_su3dslash_wilson_3d(u, psi, res, isign, cb)


def pack_gauge_field(volume, u, u_tmp):
    _d().pack_gauge_field(volume, u, u_tmp)


def unpack_gauge_field(volume, u_tmp, u):
    _d().unpack_gauge_field(volume, u_tmp, u)
