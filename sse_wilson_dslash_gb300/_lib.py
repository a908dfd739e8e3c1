"""ctypes bindings of the native libraries built by ``_build.py``.

The product path fails loudly when the libraries are missing: there is no CPU
fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")

_core = None
_legacy = {}

c_int_p = ctypes.POINTER(ctypes.c_int)
GETCOORDS = ctypes.CFUNCTYPE(None, c_int_p, ctypes.c_int, ctypes.c_int)
GETLINEAR = ctypes.CFUNCTYPE(ctypes.c_int, c_int_p)
NODENUM = ctypes.CFUNCTYPE(ctypes.c_int, c_int_p)


class SolverParams(ctypes.Structure):
    """gbds_solver_params (include/gbdslash.h)."""
    _fields_ = [("kappa", ctypes.c_double), ("tol", ctypes.c_double), ("max_iter", ctypes.c_int),
                ("inner_prec", ctypes.c_int), ("inner_recon", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("outer_double_float", ctypes.c_int)]


class SolverStats(ctypes.Structure):
    """gbds_solver_stats (include/gbdslash.h)."""
    _fields_ = [("iterations", ctypes.c_int), ("cycles", ctypes.c_int), ("converged", ctypes.c_int),
                ("residual", ctypes.c_double), ("true_residual", ctypes.c_double), ("seconds", ctypes.c_double)]


class BatchItem(ctypes.Structure):
    """gbds_batch_item (include/gbdslash.h)."""
    _fields_ = [("dims", ctypes.c_int * 4), ("nrhs", ctypes.c_int), ("isign", ctypes.c_int), ("cb", ctypes.c_int),
                ("gauge", ctypes.c_void_p), ("psi", ctypes.c_void_p), ("res", ctypes.c_void_p)]


class GbdsError(RuntimeError):
    """A gbds_* call returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"gbds status {status}: {msg}")
        self.status = status


def _path(name: str) -> str:
    p = os.path.join(LIB_DIR, name)
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build the CUDA libraries first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    return p


def core() -> ctypes.CDLL:
    """libgbdslash.so with argument types declared."""
    global _core
    if _core is not None:
        return _core
    L = ctypes.CDLL(_path("libgbdslash.so"))
    vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    L.gbds_get_last_error.restype = ctypes.c_char_p
    L.gbds_kernel_launch_count.restype = ctypes.c_longlong
    L.gbds_op_create.argtypes = [ctypes.POINTER(vp), c_int_p, i, i, i]
    L.gbds_op_create_ex.argtypes = [ctypes.POINTER(vp), c_int_p, i, i, i, i, i]
    L.gbds_op_nrhs.argtypes = [vp]
    L.gbds_op_set_tensor_cores.argtypes = [vp, i]
    L.gbds_op_check.argtypes = [vp]
    L.gbds_tc_wait_selftest.argtypes = [i]
    L.gbds_op_destroy.argtypes = [vp]
    L.gbds_op_set_layout.argtypes = [vp, c_int_p, i]
    L.gbds_op_is_canonical.argtypes = [vp]
    L.gbds_op_spinor_bytes.argtypes = [vp]
    L.gbds_op_spinor_bytes.restype = sz
    L.gbds_op_gauge_bytes.argtypes = [vp]
    L.gbds_op_gauge_bytes.restype = sz
    L.gbds_op_geometry.argtypes = [vp, c_int_p, c_int_p, c_int_p]
    L.gbds_op_set_tuning.argtypes = [vp, i, i]
    L.gbds_op_num_variants.argtypes = [vp]
    L.gbds_op_get_tuning.argtypes = [vp, c_int_p, c_int_p]
    L.gbds_op_set_site_order.argtypes = [vp, i]
    L.gbds_op_get_site_order.argtypes = [vp, c_int_p]
    L.gbds_op_autotune.argtypes = [vp, vp, vp, vp, vp]
    L.gbds_op_pack_gauge.argtypes = [vp, vp, vp, vp]
    L.gbds_op_pack_spinor.argtypes = [vp, vp, i, vp, vp]
    L.gbds_op_unpack_spinor.argtypes = [vp, vp, i, vp, vp]
    L.gbds_op_dslash.argtypes = [vp, vp, vp, vp, i, i, vp]
    for n in ("gbds_legacy_set_exit_on_error", "gbds_legacy_set_gauge_cache", "gbds_legacy_set_recon",
              "gbds_legacy_set_host_access"):
        getattr(L, n).argtypes = [i]
    L.gbds_legacy_refcount.argtypes = [i, i]
    L.gbds_layout_select.argtypes = [i, c_int_p]
    L.gbds_solver_create.argtypes = [ctypes.POINTER(vp), c_int_p, ctypes.POINTER(SolverParams)]
    L.gbds_solver_destroy.argtypes = [vp]
    L.gbds_solver_set_gauge.argtypes = [vp, vp, vp]
    L.gbds_solver_apply.argtypes = [vp, vp, vp, i, vp]
    L.gbds_solver_solve.argtypes = [vp, vp, vp, ctypes.POINTER(SolverStats), vp]
    L.gbds_solver_solve_normal.argtypes = [vp, vp, vp, ctypes.POINTER(SolverStats), vp]
    L.gbds_bsolver_create.argtypes = [ctypes.POINTER(vp), c_int_p, i, ctypes.POINTER(SolverParams)]
    L.gbds_bsolver_destroy.argtypes = [vp]
    L.gbds_bsolver_set_gauge.argtypes = [vp, vp, vp]
    L.gbds_bsolver_solve.argtypes = [vp, vp, vp, ctypes.POINTER(SolverStats), vp]
    L.gbds_op_force.argtypes = [vp, vp, vp, vp, i, i, i, ctypes.c_double, i, vp, vp]
    L.gbds_op_face_bytes.argtypes = [vp]
    L.gbds_op_face_bytes.restype = sz
    L.gbds_op_pack_faces.argtypes = [vp, vp, vp, i, i, vp, vp, vp]
    L.gbds_op_dslash_halo.argtypes = [vp, vp, vp, vp, vp, vp, i, i, i, vp]
    L.gbds_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(BatchItem), i, i, i]
    L.gbds_batch_destroy.argtypes = [vp]
    L.gbds_batch_set_schedule.argtypes = [vp, i, i, i]
    L.gbds_batch_get_schedule.argtypes = [vp, c_int_p, c_int_p, c_int_p, c_int_p]
    L.gbds_batch_autotune.argtypes = [vp, vp]
    L.gbds_batch_capture_graph.argtypes = [vp, vp]
    L.gbds_batch_launch.argtypes = [vp, vp]
    _core = L
    return L


def legacy(prec: int) -> ctypes.CDLL:
    """libgbdslash32.so / libgbdslash64.so: the reference's own entry points."""
    if prec in _legacy:
        return _legacy[prec]
    core()
    L = ctypes.CDLL(_path(f"libgbdslash{prec}.so"))
    real = ctypes.c_float if prec == 32 else ctypes.c_double
    rp = ctypes.POINTER(real)
    for n in ("init_sse_su3dslash", "init_sse_su3dslash_3d"):
        getattr(L, n).argtypes = [c_int_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        getattr(L, n).restype = None
    for n in ("sse_su3dslash_wilson", "sse_su3dslash_wilson_3d"):
        getattr(L, n).argtypes = [rp, rp, rp, ctypes.c_int, ctypes.c_int]
        getattr(L, n).restype = None
    L.pack_gauge_field.argtypes = [ctypes.c_int, rp, rp]
    L.unpack_gauge_field.argtypes = [ctypes.c_int, rp, rp]
    _legacy[prec] = L
    return L


def check(status: int) -> None:
    if status != 0:
        raise GbdsError(status, core().gbds_get_last_error().decode())


def launch_count() -> int:
    return int(core().gbds_kernel_launch_count())


def canonical_callbacks(nd: int, dims):
    """C addresses of (getSiteCoords, getLinearSiteIndex, nodeNumber) for the
    QDP++ cb2 (nd=4) / cb3d (nd=3) order of ``dims`` (gbds_layout_* in
    include/gbdslash.h)."""
    L = core()
    check(L.gbds_layout_select(int(nd), (ctypes.c_int * 4)(*[int(v) for v in dims])))
    return tuple(ctypes.cast(f, ctypes.c_void_p).value for f in
                 (L.gbds_layout_site_coords, L.gbds_layout_linear_site_index, L.gbds_layout_node_number))
