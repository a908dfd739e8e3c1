"""CPU oracle for the Wilson hopping term -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker (or as the timed CPU
baseline).  The product path in ``sse_wilson_dslash_gb300`` never imports it.

Contents
--------
* seeded input generators (Gaussian spinors, random SU(3) links built the way
  ``tests/reunit.cc:184-280`` reunitarises a Gaussian matrix, near-unit links
  ``exp(i*eps*H)``), all in the reference's packed host layouts;
* the four site layouts (QDP++ cb2 / cb3d, lexicographic, arbitrary
  permutation) as ``lin_of_lex`` tables and as C callbacks;
* three restatements of the operator (``dslash_plain`` and ``PortTables`` from
  ``dslash_oracle.c``; ``dslash_numpy`` vectorised in numpy);
* a loader for the reference library compiled from its own sources by
  ``oracle/Makefile`` into ``oracle/_ref`` (where the sources exist; with the
  host's SSE on x86_64, else through the portable shim ``sse_shim/``).

Packed layouts (the reference ABI):
  spinor ``psi[V][4 spin][3 colour][2]`` in the caller's linear site order;
  gauge  ``u[V][4 mu][3 j][3 i][2]`` with ``u[s][mu][j][i] = U_mu(s)_{ij}``
  (``lib/qdp_packer_nopad.cc:15-16`` stores the transpose).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LAYOUT_CB2, LAYOUT_CB3D, LAYOUT_LEX, LAYOUT_PERM = 0, 1, 2, 3

_lib = None


def _build_if_needed(target: str) -> None:
    path = os.path.join(HERE, target)
    src = os.path.join(HERE, "dslash_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def lib() -> ctypes.CDLL:
    """Load (building on first use) ``oracle/liboracle.so``."""
    global _lib
    if _lib is not None:
        return _lib
    _build_if_needed("liboracle.so")
    L = ctypes.CDLL(os.path.join(HERE, "liboracle.so"))
    P = ctypes.POINTER
    i32p, f64p, f32p = P(ctypes.c_int), P(ctypes.c_double), P(ctypes.c_float)
    L.orc_layout_set.argtypes = [ctypes.c_int, i32p, i32p]
    L.orc_layout_set.restype = ctypes.c_int
    L.orc_layout_callback_calls.restype = ctypes.c_long
    L.orc_layout_table.argtypes = [ctypes.c_int, i32p, i32p]
    L.orc_dslash_plain.argtypes = [ctypes.c_int, i32p, i32p, f64p, f64p, f64p, ctypes.c_int, ctypes.c_int]
    L.orc_tables_new.argtypes = [ctypes.c_int, i32p, i32p]
    L.orc_tables_new.restype = ctypes.c_void_p
    L.orc_tables_free.argtypes = [ctypes.c_void_p]
    L.orc_dslash_port_f32.argtypes = [ctypes.c_void_p, f32p, f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.orc_dslash_port_f64.argtypes = [ctypes.c_void_p, f64p, f64p, f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.orc_dslash_port_range_f32.argtypes = [ctypes.c_void_p, f32p, f32p, f32p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.orc_dslash_port_range_f64.argtypes = [ctypes.c_void_p, f64p, f64p, f64p, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.orc_max_threads.restype = ctypes.c_int
    _lib = L
    return L


def _ptr(a: np.ndarray, ctype):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _dims(dims) -> np.ndarray:
    d = np.ascontiguousarray(np.asarray(dims, dtype=np.int32))
    assert d.shape == (4,)
    return d


# --------------------------------------------------------------------------
# Layouts
# --------------------------------------------------------------------------

def volume(dims) -> int:
    return int(np.prod(np.asarray(dims, dtype=np.int64)))


def layout_table(kind: int, dims) -> np.ndarray:
    """``lin_of_lex[lex]``: linear index of lexicographic site ``lex``
    (``lex = x + Lx*(y + Ly*(z + Lz*t))``) in layout ``kind``."""
    d = _dims(dims)
    out = np.empty(volume(d), dtype=np.int32)
    lib().orc_layout_table(kind, _ptr(d, ctypes.c_int), _ptr(out, ctypes.c_int))
    return out


def scrambled_table(dims, seed: int = 7) -> np.ndarray:
    """A fixed pseudo-random permutation layout (tests arbitrary callbacks)."""
    rng = np.random.default_rng(seed)
    return rng.permutation(volume(dims)).astype(np.int32)


def set_callback_layout(kind: int, dims, lin_of_lex: np.ndarray | None = None) -> None:
    """Select the layout described by the C callbacks returned by
    :func:`callbacks`."""
    d = _dims(dims)
    if kind == LAYOUT_PERM:
        t = np.ascontiguousarray(lin_of_lex, dtype=np.int32)
        rc = lib().orc_layout_set(kind, _ptr(d, ctypes.c_int), _ptr(t, ctypes.c_int))
    else:
        rc = lib().orc_layout_set(kind, _ptr(d, ctypes.c_int), None)
    if rc != 0:
        raise ValueError(f"orc_layout_set failed ({rc})")


def callbacks():
    """(getSiteCoords, getLinearSiteIndex, nodeNumber) as C function addresses."""
    L = lib()
    return tuple(ctypes.cast(f, ctypes.c_void_p).value for f in
                 (L.orc_get_site_coords, L.orc_get_linear_site_index, L.orc_node_number))


def callback_calls() -> int:
    return int(lib().orc_layout_callback_calls())


def parity_of_lex(dims, nd: int) -> np.ndarray:
    x, y, z, t = lex_coords(dims)
    return ((x + y + z + (t if nd == 4 else 0)) & 1).astype(np.int8)


def lex_coords(dims):
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    t, z, y, x = np.meshgrid(np.arange(Lt), np.arange(Lz), np.arange(Ly), np.arange(Lx), indexing="ij")
    return x.ravel(), y.ravel(), z.ravel(), t.ravel()


# --------------------------------------------------------------------------
# Generators
# --------------------------------------------------------------------------

def gaussian_spinor(rng: np.random.Generator, V: int) -> np.ndarray:
    """N(0,1) real and imaginary parts, packed ``[V][4][3][2]`` float64."""
    return rng.standard_normal((V, 4, 3, 2))


def reunitarise(a: np.ndarray) -> np.ndarray:
    """SU(3) from complex matrices ``a[..., 3, 3]`` (rows): normalise row 0,
    Gram-Schmidt row 1, row 2 = conj(row0 x row1).  Mirrors the SU(3) branch
    of ``tests/reunit.cc:184-238``."""
    r0 = a[..., 0, :]
    r0 = r0 / np.sqrt(np.sum(np.abs(r0) ** 2, axis=-1, keepdims=True))
    r1 = a[..., 1, :]
    r1 = r1 - np.sum(np.conj(r0) * r1, axis=-1, keepdims=True) * r0
    r1 = r1 / np.sqrt(np.sum(np.abs(r1) ** 2, axis=-1, keepdims=True))
    r2 = np.conj(np.cross(r0, r1))
    return np.stack([r0, r1, r2], axis=-2)


def random_su3(rng: np.random.Generator, n: int) -> np.ndarray:
    """n random SU(3) matrices ``U[n, i, j]`` (complex128)."""
    g = rng.standard_normal((n, 3, 3, 2))
    return reunitarise(g[..., 0] + 1j * g[..., 1])


def near_unit_su3(rng: np.random.Generator, n: int, eps: float = 0.3) -> np.ndarray:
    """n matrices ``exp(i*eps*H)``, H traceless Hermitian with N(0,1) entries."""
    d = rng.standard_normal((n, 3))
    od = rng.standard_normal((n, 3, 2))
    H = np.zeros((n, 3, 3), dtype=np.complex128)
    idx = np.arange(3)
    H[:, idx, idx] = d - d.mean(axis=1, keepdims=True)
    for k, (i, j) in enumerate(((0, 1), (0, 2), (1, 2))):
        H[:, i, j] = od[:, k, 0] + 1j * od[:, k, 1]
        H[:, j, i] = np.conj(H[:, i, j])
    w, vec = np.linalg.eigh(H)
    return np.einsum("nij,nj,nkj->nik", vec, np.exp(1j * eps * w), np.conj(vec))


def pack_links(U: np.ndarray) -> np.ndarray:
    """``U[V, 4, i, j]`` complex -> packed ``u[V][4][j][i][2]`` float64."""
    Ut = np.swapaxes(U, -1, -2)
    return np.ascontiguousarray(np.stack([Ut.real, Ut.imag], axis=-1))


def unpack_links(u: np.ndarray) -> np.ndarray:
    """packed ``u[V][4][j][i][2]`` -> ``U[V, 4, i, j]`` complex128."""
    c = u[..., 0].astype(np.float64) + 1j * u[..., 1].astype(np.float64)
    return np.swapaxes(c, -1, -2)


def random_gauge(rng: np.random.Generator, V: int, kind: str = "haar") -> np.ndarray:
    """Packed gauge field ``[V][4][3][3][2]`` float64 of random SU(3) links
    (``kind='haar'``) or near-unit links (``kind='near_unit'``)."""
    if kind == "haar":
        U = random_su3(rng, V * 4)
    elif kind == "near_unit":
        U = near_unit_su3(rng, V * 4)
    else:
        raise ValueError(kind)
    return pack_links(U.reshape(V, 4, 3, 3))


def make_inputs(dims, seed_gauge: int = 1234, seed_spinor: int = 5678, kind: str = "haar"):
    """Seeded packed (u, psi) in float64 for lattice ``dims``."""
    V = volume(dims)
    u = random_gauge(np.random.default_rng(seed_gauge), V, kind)
    psi = gaussian_spinor(np.random.default_rng(seed_spinor), V)
    return u, psi


# --------------------------------------------------------------------------
# Restatements of the operator
# --------------------------------------------------------------------------

def dslash_plain(nd: int, dims, lin_of_lex: np.ndarray, u: np.ndarray, psi: np.ndarray,
                 isign: int, cb: int, res: np.ndarray | None = None) -> np.ndarray:
    """FP64 plain-C restatement; writes parity ``1-cb`` sites of ``res``
    (a float64 copy of ``res`` if given, else zeros) and returns it."""
    d = _dims(dims)
    V = volume(d)
    u64 = np.ascontiguousarray(u, dtype=np.float64).reshape(V, 4, 3, 3, 2)
    p64 = np.ascontiguousarray(psi, dtype=np.float64).reshape(V, 4, 3, 2)
    out = np.zeros((V, 4, 3, 2)) if res is None else np.array(res, dtype=np.float64).reshape(V, 4, 3, 2)
    t = np.ascontiguousarray(lin_of_lex, dtype=np.int32)
    lib().orc_dslash_plain(nd, _ptr(d, ctypes.c_int), _ptr(t, ctypes.c_int), _ptr(u64, ctypes.c_double),
                           _ptr(p64, ctypes.c_double), _ptr(out, ctypes.c_double), int(isign), int(cb))
    return out


# Half-spinor projection table: (1 - gamma_mu) psi -> h0 = psi0 + a0 psi_j0, ...
_GAMMA = np.zeros((4, 4, 4), dtype=np.complex128)
for (_mu, _r, _c, _v) in [(0, 0, 3, 1j), (0, 1, 2, 1j), (0, 2, 1, -1j), (0, 3, 0, -1j),
                          (1, 0, 3, -1), (1, 1, 2, 1), (1, 2, 1, 1), (1, 3, 0, -1),
                          (2, 0, 2, 1j), (2, 1, 3, -1j), (2, 2, 0, -1j), (2, 3, 1, 1j),
                          (3, 0, 2, 1), (3, 1, 3, 1), (3, 2, 0, 1), (3, 3, 1, 1)]:
    _GAMMA[_mu, _r, _c] = _v


def gamma_matrices() -> np.ndarray:
    """DeGrand-Rossi gamma matrices ``[mu, row, col]`` (copy)."""
    return _GAMMA.copy()


def to_lex_fields(dims, lin_of_lex, u, psi):
    """Packed caller-order arrays -> lexicographic complex arrays
    ``psi[T,Z,Y,X,4,3]`` and ``U[4,T,Z,Y,X,3,3]`` (U_ij)."""
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    V = Lx * Ly * Lz * Lt
    p = np.asarray(psi, dtype=np.float64).reshape(V, 4, 3, 2)[lin_of_lex]
    P = (p[..., 0] + 1j * p[..., 1]).reshape(Lt, Lz, Ly, Lx, 4, 3)
    U = unpack_links(np.asarray(u).reshape(V, 4, 3, 3, 2)[lin_of_lex])
    U = np.moveaxis(U.reshape(Lt, Lz, Ly, Lx, 4, 3, 3), 4, 0)
    return U, P


def dslash_numpy(nd: int, dims, lin_of_lex: np.ndarray, u: np.ndarray, psi: np.ndarray,
                 isign: int, cb: int, res: np.ndarray | None = None) -> np.ndarray:
    """Vectorised numpy FP64 restatement (same contract as ``dslash_plain``)."""
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    V = Lx * Ly * Lz * Lt
    out = np.zeros((V, 4, 3, 2)) if res is None else np.array(res, dtype=np.float64).reshape(V, 4, 3, 2)
    if isign not in (1, -1):
        return out
    U, P = to_lex_fields(dims, lin_of_lex, u, psi)
    acc = np.zeros_like(P)
    axis = {0: 3, 1: 2, 2: 1, 3: 0}
    one = np.eye(4)
    for mu in range(nd):
        pm = one - isign * _GAMMA[mu]
        pp = one + isign * _GAMMA[mu]
        fwd = np.roll(P, -1, axis=axis[mu])
        acc += np.einsum("...ij,st,...tj->...si", U[mu], pm, fwd, optimize=True)
        w = np.einsum("...ji,st,...tj->...si", np.conj(U[mu]), pp, P, optimize=True)
        acc += np.roll(w, 1, axis=axis[mu])
    par = parity_of_lex(dims, nd).reshape(Lt, Lz, Ly, Lx)
    sel = (par == 1 - cb).ravel()
    flat = acc.reshape(V, 4, 3)
    target = lin_of_lex[sel]
    out[target, ..., 0] = flat[sel].real
    out[target, ..., 1] = flat[sel].imag
    return out


class PortTables:
    """Table-driven half-spinor restatement (the CPU baseline): site table and
    neighbour tables built once per layout like ``make_shift_tables``
    (``lib/shift_tables_scalar.c:191-305``), then OpenMP over target sites."""

    def __init__(self, nd: int, dims, lin_of_lex: np.ndarray):
        d = _dims(dims)
        t = np.ascontiguousarray(lin_of_lex, dtype=np.int32)
        self._h = lib().orc_tables_new(nd, _ptr(d, ctypes.c_int), _ptr(t, ctypes.c_int))
        if not self._h:
            raise MemoryError("orc_tables_new failed")
        self.nd, self.dims, self.V = nd, tuple(int(v) for v in d), volume(d)

    def apply(self, u: np.ndarray, psi: np.ndarray, res: np.ndarray, isign: int, cb: int,
              nthreads: int | None = None) -> None:
        """res (float32 or float64, caller order) <- D psi on parity 1-cb."""
        n = max_threads() if nthreads is None else nthreads
        if res.dtype == np.float32:
            lib().orc_dslash_port_f32(self._h, _ptr(u, ctypes.c_float), _ptr(psi, ctypes.c_float),
                                      _ptr(res, ctypes.c_float), int(isign), int(cb), int(n))
        else:
            lib().orc_dslash_port_f64(self._h, _ptr(u, ctypes.c_double), _ptr(psi, ctypes.c_double),
                                      _ptr(res, ctypes.c_double), int(isign), int(cb), int(n))

    def apply_range(self, u, psi, res, isign: int, cb: int, first: int, count: int,
                    nthreads: int | None = None) -> None:
        """Only target sites [first, first+count) in traversal order."""
        n = max_threads() if nthreads is None else nthreads
        f = lib().orc_dslash_port_range_f32 if res.dtype == np.float32 else lib().orc_dslash_port_range_f64
        ct = ctypes.c_float if res.dtype == np.float32 else ctypes.c_double
        f(self._h, _ptr(u, ct), _ptr(psi, ct), _ptr(res, ct), int(isign), int(cb), int(first), int(count), int(n))

    def close(self):
        if self._h:
            lib().orc_tables_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def max_threads() -> int:
    return int(lib().orc_max_threads())


# --------------------------------------------------------------------------
# Metrics used by the parity tests
# --------------------------------------------------------------------------

def site_rel_err(got: np.ndarray, ref: np.ndarray, sites: np.ndarray) -> float:
    """max over ``sites`` of ||got_site - ref_site|| / ||ref_site||."""
    V = ref.reshape(-1, 24).shape[0]
    g = np.asarray(got, dtype=np.float64).reshape(V, 24)[sites]
    r = np.asarray(ref, dtype=np.float64).reshape(V, 24)[sites]
    num = np.sqrt(np.sum((g - r) ** 2, axis=1))
    den = np.sqrt(np.sum(r ** 2, axis=1))
    return float(np.max(num / np.maximum(den, 1e-300)))


def target_sites(nd: int, dims, lin_of_lex: np.ndarray, cb: int) -> np.ndarray:
    """Caller linear indices of the sites written for source checkerboard cb."""
    par = parity_of_lex(dims, nd)
    return np.asarray(lin_of_lex)[par == 1 - cb]


# --------------------------------------------------------------------------
# The reference library built from its own sources
# --------------------------------------------------------------------------

def _ref_path(prec: int, shim: bool) -> str:
    return os.path.join(HERE, "_ref", f"libref{prec}{'_shim' if shim else ''}.so")


def reference_available(prec: int, shim: bool = False) -> bool:
    """The reference library built from its sources: ``shim=False`` the build
    for this host (native SSE on x86_64, the portable SSE shim elsewhere),
    ``shim=True`` the shim build made beside the native one on x86_64."""
    return os.path.exists(_ref_path(prec, shim))


class Reference:
    """ctypes binding of the reference scalar library (``oracle/_ref``)."""

    def __init__(self, prec: int, shim: bool = False):
        path = _ref_path(prec, shim)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.prec = prec
        self.real = ctypes.c_float if prec == 32 else ctypes.c_double
        self.np_real = np.float32 if prec == 32 else np.float64
        L = ctypes.CDLL(path)
        rp = ctypes.POINTER(self.real)
        for nm in ("init_sse_su3dslash", "init_sse_su3dslash_3d"):
            getattr(L, nm).argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for nm in ("sse_su3dslash_wilson", "sse_su3dslash_wilson_3d"):
            getattr(L, nm).argtypes = [rp, rp, rp, ctypes.c_int, ctypes.c_int]
        L.pack_gauge_field.argtypes = [ctypes.c_int, rp, rp]
        L.unpack_gauge_field.argtypes = [ctypes.c_int, rp, rp]
        self.L = L

    def init(self, nd: int, dims, kind: int, lin_of_lex=None):
        set_callback_layout(kind, dims, lin_of_lex)
        d = (ctypes.c_int * 4)(*[int(v) for v in dims])
        f = self.L.init_sse_su3dslash if nd == 4 else self.L.init_sse_su3dslash_3d
        f(d, *callbacks())

    def free(self, nd: int):
        (self.L.free_sse_su3dslash if nd == 4 else self.L.free_sse_su3dslash_3d)()

    def apply(self, nd: int, u: np.ndarray, psi: np.ndarray, res: np.ndarray, isign: int, cb: int):
        rp = ctypes.POINTER(self.real)
        for a in (u, psi, res):
            assert a.dtype == self.np_real and a.flags["C_CONTIGUOUS"]
        f = self.L.sse_su3dslash_wilson if nd == 4 else self.L.sse_su3dslash_wilson_3d
        f(u.ctypes.data_as(rp), psi.ctypes.data_as(rp), res.ctypes.data_as(rp), int(isign), int(cb))
