"""Device-resident Dslash on torch CUDA tensors, through the extended C ABI
(``gbds_op_*`` in include/gbdslash.h).

Torch is used only for device memory and streams; the work is done by the
library's own kernels.  Fields in the internal layout are plain uint8 CUDA
tensors of ``spinor_bytes`` / ``gauge_bytes``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _dptr(t) -> int:
    if not t.is_cuda:
        raise TypeError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise TypeError("expected a contiguous tensor")
    return t.data_ptr()


def _stream(stream):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


class DslashOperator:
    """Wilson hopping term on one lattice.

    dims: (Lx, Ly, Lz, Lt); nd: 4 (4D, QDP++ cb2 order) or 3 (spatial, cb3d);
    prec: 32 or 64; recon: 18 or 12 (12-real links, SU(3) only).
    spinor_format "double_float" (prec 64, one rhs): FP64 fields held and
    computed as hi + lo FP32 pairs on the FP32 pipes.
    """

    FORMATS = {"native": 0, "bf16": 1, "f16": 2, "f32_pairs": 3, "double_float": 4}

    def __init__(self, dims, nd: int = 4, prec: int = 32, recon: int = 18, device=None, nrhs: int = 1,
                 spinor_format: str = "native"):
        import torch
        self.dims = tuple(int(v) for v in dims)
        self.nd, self.prec, self.recon, self.nrhs = nd, prec, recon, nrhs
        self.spinor_format = spinor_format
        self.device = torch.device("cuda" if device is None else device)
        L = _lib.core()
        h = ctypes.c_void_p()
        d = (ctypes.c_int * 4)(*self.dims)
        _lib.check(L.gbds_op_create_ex(ctypes.byref(h), d, nd, prec, recon, nrhs, self.FORMATS[spinor_format]))
        self._h = h
        V, Vh, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(L.gbds_op_geometry(h, ctypes.byref(V), ctypes.byref(Vh), ctypes.byref(st)))
        self.volume, self.volume_cb, self.stride = V.value, Vh.value, st.value
        self.spinor_bytes = int(L.gbds_op_spinor_bytes(h))
        self.gauge_bytes = int(L.gbds_op_gauge_bytes(h))
        self.real_dtype = torch.float32 if prec == 32 else torch.float64
        # packed dtype of the gauge field (FP32 for the generalised formats)

    def close(self):
        if getattr(self, "_h", None):
            _lib.core().gbds_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- layout ----------------------------------------------------------------
    def set_layout(self, site_table) -> None:
        """Caller site order: ``site_table[i]`` = caller index of internal site i
        (None = canonical)."""
        if site_table is None:
            _lib.check(_lib.core().gbds_op_set_layout(self._h, None, 0))
            return
        t = np.ascontiguousarray(site_table, dtype=np.int32)
        _lib.check(_lib.core().gbds_op_set_layout(self._h, t.ctypes.data_as(_lib.c_int_p), int(t.size)))

    @property
    def canonical(self) -> bool:
        return bool(_lib.core().gbds_op_is_canonical(self._h))

    def set_tensor_cores(self, on: bool = True) -> None:
        """Colour multiply on the tensor cores (16-bit formats, nrhs 16 or 32)."""
        _lib.check(_lib.core().gbds_op_set_tensor_cores(self._h, 1 if on else 0))

    def check(self) -> None:
        """Synchronise; raise if a tensor-core launch timed out."""
        _lib.check(_lib.core().gbds_op_check(self._h))

    def set_tuning(self, threads: int, variant: int = 0) -> None:
        _lib.check(_lib.core().gbds_op_set_tuning(self._h, int(threads), int(variant)))

    def tuning(self):
        b, v = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.core().gbds_op_get_tuning(self._h, ctypes.byref(b), ctypes.byref(v)))
        return b.value, v.value

    def set_site_order(self, zblock: int) -> None:
        """Site order of the multi-RHS kernels: z slabs of ``zblock`` planes
        (a divisor of Lz), 0 the natural order, -1 the default."""
        _lib.check(_lib.core().gbds_op_set_site_order(self._h, int(zblock)))

    def site_order(self) -> int:
        z = ctypes.c_int()
        _lib.check(_lib.core().gbds_op_get_site_order(self._h, ctypes.byref(z)))
        return z.value

    def autotune(self, gauge, psi, scratch, stream=None):
        """Pick the fastest launch configuration on these fields (scratch is overwritten)."""
        _lib.check(_lib.core().gbds_op_autotune(self._h, ctypes.c_void_p(_dptr(gauge)), ctypes.c_void_p(_dptr(psi)),
                                                ctypes.c_void_p(_dptr(scratch)), _stream(stream)))
        return self.tuning()

    @property
    def num_variants(self) -> int:
        return int(_lib.core().gbds_op_num_variants(self._h))

    # -- fields ----------------------------------------------------------------
    def new_spinor(self):
        import torch
        return torch.empty(self.spinor_bytes, dtype=torch.uint8, device=self.device)

    def new_gauge(self):
        import torch
        return torch.empty(self.gauge_bytes, dtype=torch.uint8, device=self.device)

    def pack_gauge(self, u_packed, out=None, stream=None):
        """Packed device gauge ``[V][4][3][3][2]`` -> internal layout."""
        out = self.new_gauge() if out is None else out
        self._check_real(u_packed, self.volume * 72)
        _lib.check(_lib.core().gbds_op_pack_gauge(self._h, ctypes.c_void_p(_dptr(u_packed)),
                                                  ctypes.c_void_p(_dptr(out)), _stream(stream)))
        return out

    def pack_spinor(self, psi_packed, parity: int, out=None, stream=None):
        """Packed device spinor ``[nrhs][V][4][3][2]`` (checkerboard ``parity``) -> internal."""
        out = self.new_spinor() if out is None else out
        self._check_real(psi_packed, self.volume * 24 * self.nrhs)
        _lib.check(_lib.core().gbds_op_pack_spinor(self._h, ctypes.c_void_p(_dptr(psi_packed)), int(parity),
                                                   ctypes.c_void_p(_dptr(out)), _stream(stream)))
        return out

    def unpack_spinor(self, spinor, parity: int, psi_packed, stream=None):
        """Internal spinor -> the checkerboard ``parity`` sites of a packed array."""
        self._check_real(psi_packed, self.volume * 24 * self.nrhs)
        _lib.check(_lib.core().gbds_op_unpack_spinor(self._h, ctypes.c_void_p(_dptr(spinor)), int(parity),
                                                     ctypes.c_void_p(_dptr(psi_packed)), _stream(stream)))
        return psi_packed

    def apply(self, gauge, psi, isign: int, cb: int, out=None, stream=None):
        """out (checkerboard 1-cb) = Dslash psi (checkerboard cb), internal layout."""
        out = self.new_spinor() if out is None else out
        for t, n in ((gauge, self.gauge_bytes), (psi, self.spinor_bytes), (out, self.spinor_bytes)):
            if t.numel() * t.element_size() < n:
                raise ValueError("field buffer too small")
        _lib.check(_lib.core().gbds_op_dslash(self._h, ctypes.c_void_p(_dptr(gauge)), ctypes.c_void_p(_dptr(psi)),
                                              ctypes.c_void_p(_dptr(out)), int(isign), int(cb), _stream(stream)))
        return out

    def force(self, gauge, psi, chi, isign: int, cb: int, out, mode: int = 1, coef: float = 1.0,
              accumulate: bool = False, stream=None):
        """dL/dU for L = Re <chi, Dslash(isign) psi> (psi on cb, chi on 1-cb,
        internal fields) into the packed gauge-layout tensor ``out``: mode 0
        the complex gradient G, mode 1 the su(3) force TA(G U^+)."""
        self._check_real(out, self.volume * 72)
        _lib.check(_lib.core().gbds_op_force(self._h, ctypes.c_void_p(_dptr(gauge)), ctypes.c_void_p(_dptr(psi)),
                                             ctypes.c_void_p(_dptr(chi)), int(isign), int(cb), int(mode), float(coef),
                                             1 if accumulate else 0, ctypes.c_void_p(_dptr(out)), _stream(stream)))
        return out

    # -- time direction split across ranks (gbds_op_pack_faces / _dslash_halo) ---
    HALO_PARTS = {"all": 0, "interior": 1, "boundary": 2}

    @property
    def face_bytes(self) -> int:
        """Bytes of one face buffer (one checkerboard of a time slice, 12 reals a site)."""
        return int(_lib.core().gbds_op_face_bytes(self._h))

    def new_face(self):
        import torch
        return torch.empty(self.face_bytes, dtype=torch.uint8, device=self.device)

    def pack_faces(self, gauge, psi, isign: int, cb: int, to_prev, to_next, stream=None):
        """Send buffers of the source psi (checkerboard cb) when t is split
        across ranks: to_prev = (1 - isign g_t) psi on the first time slice,
        to_next = U_t^+ (1 + isign g_t) psi on the last one."""
        for t in (to_prev, to_next):
            if t.numel() * t.element_size() < self.face_bytes:
                raise ValueError("face buffer too small")
        _lib.check(_lib.core().gbds_op_pack_faces(self._h, ctypes.c_void_p(_dptr(gauge)), ctypes.c_void_p(_dptr(psi)),
                                                  int(isign), int(cb), ctypes.c_void_p(_dptr(to_prev)),
                                                  ctypes.c_void_p(_dptr(to_next)), _stream(stream)))

    def apply_halo(self, gauge, psi, from_prev, from_next, isign: int, cb: int, out=None, part: str = "all",
                   stream=None):
        """out (checkerboard 1-cb) = Dslash psi with the t hops across the slab
        boundaries taken from the received faces; part 'interior' needs none."""
        out = self.new_spinor() if out is None else out
        fp = ctypes.c_void_p(_dptr(from_prev)) if from_prev is not None else None
        fn = ctypes.c_void_p(_dptr(from_next)) if from_next is not None else None
        _lib.check(_lib.core().gbds_op_dslash_halo(self._h, ctypes.c_void_p(_dptr(gauge)), ctypes.c_void_p(_dptr(psi)),
                                                   fp, fn, ctypes.c_void_p(_dptr(out)), int(isign), int(cb),
                                                   self.HALO_PARTS[part], _stream(stream)))
        return out

    def _check_real(self, t, n):
        if t.dtype != self.real_dtype:
            raise TypeError(f"expected {self.real_dtype}")
        if t.numel() < n:
            raise ValueError("packed array too small")

    # -- flop / byte accounting ----------------------------------------------------
    @property
    def flops_per_site(self) -> int:
        """Standard count: 1320 (4D), 984 (3D) per output site."""
        return 1320 if self.nd == 4 else 984

    @property
    def bytes_per_site(self) -> int:
        """Compulsory HBM bytes per output site and right-hand side: 2 spinors +
        2*nd links shared by the nrhs right-hand sides."""
        real = 4 if self.prec == 32 else 8
        spinor = {"native": 24 * real, "bf16": 48, "f16": 52, "f32_pairs": 96, "double_float": 192}[self.spinor_format]
        return 2 * spinor + 2 * self.nd * self.recon * real / self.nrhs


class WilsonSolver:
    """Even-odd preconditioned Wilson solve M x = b on the even sites,
    M = 1 - kappa^2 D_eo D_oe, by CG on M^+M (gbds_solver_* in
    include/gbdslash.h).  Fields are FP64 torch CUDA tensors in the reference's
    packed layout ``[V][4][3][2]``, QDP++ cb2 order.

    inner_prec 64: all-FP64 CG.  inner_prec 32: FP32 CG inside FP64 defect
    correction (residual, solution update and global norms in FP64).
    outer_double_float: the outer residual's operator in double-float
    arithmetic on the FP32 pipes instead of FP64."""

    def __init__(self, dims, kappa: float, tol: float = 1e-10, max_iter: int = 10000, inner_prec: int = 32,
                 inner_recon: int = 12, inner_tol: float = 1e-5, outer_double_float: bool = False):
        self.dims = tuple(int(v) for v in dims)
        self.volume = int(np.prod(self.dims))
        p = _lib.SolverParams(kappa, tol, max_iter, inner_prec, inner_recon, inner_tol, int(outer_double_float))
        h = ctypes.c_void_p()
        _lib.check(_lib.core().gbds_solver_create(ctypes.byref(h), (ctypes.c_int * 4)(*self.dims), ctypes.byref(p)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.core().gbds_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, t, n):
        import torch
        if t.dtype != torch.float64 or t.numel() < n:
            raise ValueError(f"expected a float64 CUDA tensor with at least {n} elements")

    def set_gauge(self, u_packed, stream=None):
        self._check(u_packed, self.volume * 72)
        _lib.check(_lib.core().gbds_solver_set_gauge(self._h, ctypes.c_void_p(_dptr(u_packed)), _stream(stream)))

    def apply(self, x, y, dagger: bool = False, stream=None):
        """y_even = M x_even (or M^+)."""
        self._check(x, self.volume * 24)
        self._check(y, self.volume * 24)
        _lib.check(_lib.core().gbds_solver_apply(self._h, ctypes.c_void_p(_dptr(x)), ctypes.c_void_p(_dptr(y)),
                                                 1 if dagger else 0, _stream(stream)))
        return y

    def solve(self, b, x, stream=None, normal: bool = False) -> dict:
        """M x = b, or with normal=True M^+ M x = b (b then the normal-equation right-hand side)."""
        self._check(b, self.volume * 24)
        self._check(x, self.volume * 24)
        st = _lib.SolverStats()
        f = _lib.core().gbds_solver_solve_normal if normal else _lib.core().gbds_solver_solve
        _lib.check(f(self._h, ctypes.c_void_p(_dptr(b)), ctypes.c_void_p(_dptr(x)), ctypes.byref(st), _stream(stream)))
        return {k: getattr(st, k) for k, _ in st._fields_}


class BatchedWilsonSolver:
    """``nrhs`` (2, 4, 8, 16 or 32) independent solves M x_q = b_q on one gauge
    field (gbds_bsolver_* in include/gbdslash.h): the FP32 inner CGs advance
    together on the multi-RHS operator, the FP64 defect correction runs per
    right-hand side (outer_double_float: its operator in double-float).
    b, x: FP64 CUDA tensors ``[nrhs][V][4][3][2]``."""

    def __init__(self, dims, nrhs: int, kappa: float, tol: float = 1e-10, max_iter: int = 10000,
                 inner_recon: int = 12, inner_tol: float = 1e-5, outer_double_float: bool = False):
        self.dims = tuple(int(v) for v in dims)
        self.volume = int(np.prod(self.dims))
        self.nrhs = int(nrhs)
        p = _lib.SolverParams(kappa, tol, max_iter, 32, inner_recon, inner_tol, int(outer_double_float))
        h = ctypes.c_void_p()
        _lib.check(_lib.core().gbds_bsolver_create(ctypes.byref(h), (ctypes.c_int * 4)(*self.dims), self.nrhs,
                                                   ctypes.byref(p)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.core().gbds_bsolver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_gauge(self, u_packed, stream=None):
        import torch
        if u_packed.dtype != torch.float64 or u_packed.numel() < self.volume * 72:
            raise ValueError("expected the FP64 packed gauge field")
        _lib.check(_lib.core().gbds_bsolver_set_gauge(self._h, ctypes.c_void_p(_dptr(u_packed)), _stream(stream)))

    def solve(self, b, x, stream=None) -> list:
        import torch
        n = self.nrhs * self.volume * 24
        for t in (b, x):
            if t.dtype != torch.float64 or t.numel() < n:
                raise ValueError(f"expected float64 CUDA tensors with at least {n} elements")
        st = (_lib.SolverStats * self.nrhs)()
        _lib.check(_lib.core().gbds_bsolver_solve(self._h, ctypes.c_void_p(_dptr(b)), ctypes.c_void_p(_dptr(x)), st,
                                                  _stream(stream)))
        return [{k: getattr(s, k) for k, _ in s._fields_} for s in st]


class DslashBatch:
    """Several lattices applied by one persistent launch (gbds_batch_* in
    include/gbdslash.h).  ``items``: list of dicts with keys op
    (a DslashOperator of the item's dims/nrhs, prec 32, nd 4), gauge, psi, res
    (internal fields of that op), isign, cb.  Fields must stay alive."""

    def __init__(self, items, recon: int = 18, spinor_format: str = "native"):
        arr = (_lib.BatchItem * len(items))()
        for k, it in enumerate(items):
            op = it["op"]
            arr[k].dims = (ctypes.c_int * 4)(*op.dims)
            arr[k].nrhs = op.nrhs
            arr[k].isign = int(it["isign"])
            arr[k].cb = int(it["cb"])
            arr[k].gauge = _dptr(it["gauge"])
            arr[k].psi = _dptr(it["psi"])
            arr[k].res = _dptr(it["res"])
        h = ctypes.c_void_p()
        _lib.check(_lib.core().gbds_batch_create(ctypes.byref(h), arr, len(items), int(recon),
                                                 DslashOperator.FORMATS[spinor_format]))
        self._h = h
        self._items = items

    def close(self):
        if getattr(self, "_h", None):
            _lib.core().gbds_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def schedule(self):
        v = [ctypes.c_int() for _ in range(4)]
        _lib.check(_lib.core().gbds_batch_get_schedule(self._h, *[ctypes.byref(x) for x in v]))
        return dict(tile_threads=v[0].value, resident_ctas=v[1].value, order=v[2].value, tiles=v[3].value)

    def set_schedule(self, tile_threads: int, resident_ctas: int, order: int):
        _lib.check(_lib.core().gbds_batch_set_schedule(self._h, tile_threads, resident_ctas, order))

    def autotune(self, stream=None):
        _lib.check(_lib.core().gbds_batch_autotune(self._h, _stream(stream)))
        return self.schedule()

    def capture_graph(self, stream):
        _lib.check(_lib.core().gbds_batch_capture_graph(self._h, _stream(stream)))

    def launch(self, stream=None):
        _lib.check(_lib.core().gbds_batch_launch(self._h, _stream(stream)))
