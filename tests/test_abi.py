"""The C-ABI libraries load and export every symbol the headers declare, and
the host-side logic of the drop-in behaves like the reference.  CPU only: no
call here launches a kernel."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
INCLUDE = os.path.join(ROOT, "include")

REFERENCE_API = ["init_sse_su3dslash", "free_sse_su3dslash", "sse_su3dslash_wilson",
                 "sse_su3dslash_prepost_receives", "init_sse_su3dslash_3d", "free_sse_su3dslash_3d",
                 "sse_su3dslash_wilson_3d", "pack_gauge_field", "unpack_gauge_field"]


@pytest.fixture(scope="session")
def libs():
    from sse_wilson_dslash_gb300 import _build
    return _build.build()


def declared(header):
    txt = open(os.path.join(INCLUDE, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(\w+)\s*\([^;{]*\)\s*;", txt)) - {"if", "while", "sizeof"})


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_core_exports_everything_in_gbdslash_h(libs):
    names = declared("gbdslash.h")
    assert len(names) > 30
    missing = set(names) - exported(libs["core"])
    assert not missing, missing


@pytest.mark.parametrize("prec", [32, 64])
def test_dropin_exports_reference_api(libs, prec):
    ex = exported(libs[f"legacy{prec}"])
    decl = set(declared("sse_dslash.h")) | set(declared("sse_dslash_3d.h"))
    assert decl == set(REFERENCE_API)
    assert set(REFERENCE_API) <= ex
    ctypes.CDLL(libs[f"legacy{prec}"])  # loads and resolves libgbdslash.so via $ORIGIN


def test_op_create_validation(libs):
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    h = ctypes.c_void_p()
    for dims, nd, prec, recon, ok in [((4, 4, 4, 4), 4, 32, 18, True), ((4, 4, 4, 3), 4, 32, 18, False),
                                      ((4, 4, 4, 3), 3, 64, 12, True), ((3, 4, 4, 4), 3, 32, 18, False),
                                      ((4, 4, 4, 4), 5, 32, 18, False), ((4, 4, 4, 4), 4, 16, 18, False),
                                      ((4, 4, 4, 4), 4, 32, 9, False), ((0, 4, 4, 4), 4, 32, 18, False)]:
        d = (ctypes.c_int * 4)(*dims)
        rc = L.gbds_op_create(ctypes.byref(h), d, nd, prec, recon)
        assert (rc == 0) == ok, (dims, nd, prec, recon, L.gbds_get_last_error())
        if ok:
            V, Vh, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            assert L.gbds_op_geometry(h, ctypes.byref(V), ctypes.byref(Vh), ctypes.byref(st)) == 0
            assert V.value == np.prod(dims) and Vh.value * 2 == V.value and st.value % 64 == 0 and st.value >= Vh.value
            real = prec // 8
            assert L.gbds_op_spinor_bytes(h) == 24 * real * st.value
            assert L.gbds_op_gauge_bytes(h) == 2 * nd * recon * real * st.value
            assert L.gbds_op_set_tuning(h, 96, 0) == 0 and L.gbds_op_set_tuning(h, 100, 0) != 0
            nv = L.gbds_op_num_variants(h)
            assert nv >= 2 and L.gbds_op_set_tuning(h, 0, nv - 1) == 0 and L.gbds_op_set_tuning(h, 0, nv) != 0
            L.gbds_op_destroy(h)
        else:
            assert L.gbds_get_last_error()


def test_spinor_formats_and_their_variants(libs):
    """Formats 0..3 (FP32, BF16, half + norm, FP32 spin pairs) with several
    right-hand sides: field sizes, kernel variants, tensor-core eligibility
    (16-bit formats only); no device work."""
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    h = ctypes.c_void_p()
    d = (ctypes.c_int * 4)(4, 4, 4, 4)
    for fmt, nbytes, nv in ((0, 96, 5), (1, 48, 5), (2, 52, 5), (3, 96, 5)):
        assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 32, 18, 32, fmt) == 0, L.gbds_get_last_error()
        V, Vh, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert L.gbds_op_geometry(h, ctypes.byref(V), ctypes.byref(Vh), ctypes.byref(st)) == 0
        assert L.gbds_op_spinor_bytes(h) == nbytes * st.value * 32
        assert L.gbds_op_num_variants(h) == nv
        # default from 16 rhs on: variant 4 (two rhs a thread, prefetched) for
        # the 16-bit formats, 3 (two rhs a thread) for both FP32 layouts
        blk, var = ctypes.c_int(), ctypes.c_int()
        assert L.gbds_op_get_tuning(h, ctypes.byref(blk), ctypes.byref(var)) == 0
        assert var.value == {0: 3, 1: 4, 2: 4, 3: 3}[fmt]
        if fmt in (0, 3):
            assert L.gbds_op_set_tensor_cores(h, 1) != 0
        L.gbds_op_destroy(h)
    # 8 rhs: the plain kernel, except half + norm (the fully packed one)
    for fmt, want in ((0, 0), (1, 0), (2, 2), (3, 0)):
        assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 32, 18, 8, fmt) == 0
        blk, var = ctypes.c_int(), ctypes.c_int()
        assert L.gbds_op_get_tuning(h, ctypes.byref(blk), ctypes.byref(var)) == 0 and var.value == want, fmt
        L.gbds_op_destroy(h)
    assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 32, 18, 4, 4) != 0
    # the non-native formats need prec 32 and nd 4
    assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 64, 18, 1, 3) != 0


def test_set_layout_rejects_non_permutations(libs):
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    h = ctypes.c_void_p()
    assert L.gbds_op_create(ctypes.byref(h), (ctypes.c_int * 4)(2, 2, 2, 2), 4, 32, 18) == 0
    bad = np.zeros(16, np.int32)
    assert L.gbds_op_set_layout(h, bad.ctypes.data_as(_lib.c_int_p), 16) == 1
    short = np.arange(8, dtype=np.int32)
    assert L.gbds_op_set_layout(h, short.ctypes.data_as(_lib.c_int_p), 8) == 1
    ident = np.arange(16, dtype=np.int32)  # identity: canonical, no device copy needed
    assert L.gbds_op_set_layout(h, ident.ctypes.data_as(_lib.c_int_p), 16) == 0
    assert L.gbds_op_is_canonical(h) == 1
    L.gbds_op_destroy(h)


@pytest.mark.parametrize("prec", [32, 64])
def test_pack_gauge_field_matches_reference_semantics(libs, prec):
    """pack_gauge_field: u[mu][cb][ix] -> u_tmp[cb][ix][mu] (lib/packer_nopad.c:29-45);
    unpack_gauge_field copies index for index (lib/packer_nopad.c:47-69)."""
    from sse_wilson_dslash_gb300.legacy import SSEDslash
    d = SSEDslash(prec)
    vol = 6
    rng = np.random.default_rng(3)
    u = rng.standard_normal((4, 2, vol, 3, 3, 2)).astype(d.dtype)
    out = np.zeros((2, vol, 4, 3, 3, 2), d.dtype)
    d.pack_gauge_field(vol, u, out)
    assert np.array_equal(out, np.transpose(u, (1, 2, 0, 3, 4, 5)))
    back = np.zeros_like(u)
    d.unpack_gauge_field(vol, out, back)
    assert np.array_equal(back.ravel(), out.ravel())
    import oracle as O
    if O.reference_available(prec):
        R = O.Reference(prec)
        ref = np.zeros_like(out)
        rp = ctypes.POINTER(R.real)
        R.L.pack_gauge_field(vol, u.ctypes.data_as(rp), ref.ctypes.data_as(rp))
        assert np.array_equal(ref, out)
        rb = np.zeros_like(u)
        R.L.unpack_gauge_field(vol, out.ctypes.data_as(rp), rb.ctypes.data_as(rp))
        assert np.array_equal(rb, back)


def _child(code):
    env = dict(os.environ, PYTHONPATH=ROOT, CUDA_VISIBLE_DEVICES="")
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)


@pytest.mark.parametrize("prec,nd,dims,msg", [(32, 4, (4, 4, 3, 4), "latt_size[2]=3"),
                                               (64, 4, (5, 4, 4, 4), "latt_size[0]=5"),
                                               (32, 3, (4, 3, 4, 4), "latt_size[1]=3")])
def test_init_with_odd_dims_exits_like_reference(libs, prec, nd, dims, msg):
    code = f"""
from sse_wilson_dslash_gb300.legacy import SSEDslash
import oracle as O
d = SSEDslash({prec})
O.set_callback_layout(O.LAYOUT_LEX, {dims})
gc, gl, nn = O.callbacks()
d.{'init_sse_su3dslash' if nd == 4 else 'init_sse_su3dslash_3d'}({dims}, gc, gl, nn)
print("not reached")
"""
    r = _child(code)
    assert r.returncode == 1, r.stdout + r.stderr
    assert msg in r.stderr and "not reached" not in r.stdout


def test_init_odd_time_extent_is_fine_in_3d_validation(libs):
    """3D checks only extents 0..2 (lib/sse_su3dslash_32bit_scalar_3d.c:95-102);
    with exit disabled and no GPU the init fails later, at allocation."""
    code = """
from sse_wilson_dslash_gb300 import legacy
import oracle as O
legacy.set_exit_on_error(False)
d = legacy.SSEDslash(32)
O.set_callback_layout(O.LAYOUT_CB3D, (4, 4, 4, 3))
gc, gl, nn = O.callbacks()
d.init_sse_su3dslash_3d((4, 4, 4, 3), gc, gl, nn)
print("calls", O.callback_calls(), "ref", legacy.refcount(32, 3))
"""
    r = _child(code)
    assert r.returncode == 0, r.stderr
    assert "odd" not in r.stderr and "even" not in r.stderr
    # every site's index was read through the callbacks before allocation
    assert "calls 384" in r.stdout, r.stdout


def test_no_exit_mode_and_uninitialised_apply(libs):
    code = """
import numpy as np
from sse_wilson_dslash_gb300 import legacy
import oracle as O
legacy.set_exit_on_error(False)
d = legacy.SSEDslash(32)
O.set_callback_layout(O.LAYOUT_LEX, (4, 4, 3, 4))
gc, gl, nn = O.callbacks()
d.init_sse_su3dslash((4, 4, 3, 4), gc, gl, nn)
print("ref", legacy.refcount(32, 4))
u = np.zeros((48, 4, 3, 3, 2), np.float32); p = np.zeros((48, 4, 3, 2), np.float32); r = p.copy()
d.sse_su3dslash_wilson(u, p, r, 1, 0)      # not initialised: message, no crash
d.sse_su3dslash_wilson(u, p, r, 7, 0)      # bad isign: silent no-op
d.free_sse_su3dslash(); d.free_sse_su3dslash()   # free when uninitialised: no-op
d.sse_su3dslash_prepost_receives()
print("done")
"""
    r = _child(code)
    assert r.returncode == 0, r.stderr
    assert "ref 0" in r.stdout and "done" in r.stdout
    assert "latt_size[2]=3" in r.stderr
    assert r.stderr.count("called before init") == 1


def test_bad_layout_callbacks_rejected(libs):
    code = """
from sse_wilson_dslash_gb300 import legacy
legacy.set_exit_on_error(False)
d = legacy.SSEDslash(64)
d.init_sse_su3dslash((2, 2, 2, 2), None, lambda c: 0)
print("ref", legacy.refcount(64, 4))
d.init_sse_su3dslash((2, 2, 2, 2), lambda c, n, l: None, lambda c: c[0] + 2 * (c[1] + 2 * (c[2] + 2 * c[3])))
print("ref", legacy.refcount(64, 4))
"""
    r = _child(code)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("ref 0") == 2
    assert "one-to-one" in r.stderr and "not the inverse" in r.stderr


def test_split_t_entry_points_validate_before_any_device_work(libs):
    """gbds_op_face_bytes / gbds_op_pack_faces / gbds_op_dslash_halo: face
    size, unsupported operators, bad arguments and the silent isign no-op are
    all decided on the host."""
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    vp = ctypes.c_void_p
    h = vp()
    d = (ctypes.c_int * 4)(8, 4, 6, 10)
    assert L.gbds_op_create(ctypes.byref(h), d, 4, 32, 18) == 0
    # one checkerboard of a time slice: 8 * 4 * 6 / 2 half spinors of 12 reals
    assert L.gbds_op_face_bytes(h) == 96 * 12 * 4
    a = vp(1 << 20)  # 16-byte aligned stand-ins: nothing below dereferences them
    bad = vp((1 << 20) + 8)
    assert L.gbds_op_pack_faces(h, a, a, 0, 0, a, a, None) == 0          # isign 0: no-op
    assert L.gbds_op_pack_faces(h, a, a, 1, 2, a, a, None) == 1          # cb
    assert L.gbds_op_pack_faces(h, a, a, 1, 0, None, a, None) == 1       # NULL face
    assert L.gbds_op_pack_faces(h, a, a, 1, 0, bad, a, None) == 1        # misaligned
    assert L.gbds_op_dslash_halo(h, a, a, a, a, a, 1, 0, 7, None) == 1   # part
    assert L.gbds_op_dslash_halo(h, a, a, None, a, a, 1, 0, 0, None) == 1  # faces needed
    assert L.gbds_op_dslash_halo(h, a, a, a, a, a, -2, 0, 0, None) == 0  # isign: no-op
    L.gbds_op_destroy(h)
    d64 = (ctypes.c_int * 4)(4, 4, 4, 4)
    assert L.gbds_op_create(ctypes.byref(h), d64, 4, 64, 12) == 0
    assert L.gbds_op_face_bytes(h) == 32 * 12 * 8
    L.gbds_op_destroy(h)
    # several rhs, another storage format or the 3D operator: not split
    for nd, nrhs, fmt in ((4, 8, 0), (4, 1, 1), (3, 1, 0)):
        assert L.gbds_op_create_ex(ctypes.byref(h), d64, nd, 32, 18, nrhs, fmt) == 0
        assert L.gbds_op_pack_faces(h, a, a, 1, 0, a, a, None) == 5
        assert L.gbds_op_dslash_halo(h, a, a, a, a, a, 1, 0, 0, None) == 5
        L.gbds_op_destroy(h)


def test_site_order_validation_and_defaults(libs):
    """gbds_op_set_site_order / gbds_op_get_site_order: divisors of Lz only,
    Lz itself is the natural order, single-rhs operators keep the natural
    order; the default slab is the largest divisor B of Lz whose 2 B planes
    of traffic (nrhs source and target spinors and 8 links a site) fit in
    64 MB, or the natural order when 2 Lz planes fit."""
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    h = ctypes.c_void_p()
    z = ctypes.c_int()

    def create(dims, nrhs, fmt, recon=18):
        assert L.gbds_op_create_ex(ctypes.byref(h), (ctypes.c_int * 4)(*dims), 4, 32, recon, nrhs, fmt) == 0

    def order():
        assert L.gbds_op_get_site_order(h, ctypes.byref(z)) == 0
        return z.value

    create((8, 4, 6, 10), 16, 3)
    assert order() == 0
    for zb, rc, want in ((3, 0, 3), (6, 0, 0), (1, 0, 1), (4, 1, 1), (7, 1, 1), (-2, 1, 1), (2, 0, 2), (-1, 0, 0)):
        assert L.gbds_op_set_site_order(h, zb) == rc, zb
        assert order() == want, zb
    L.gbds_op_destroy(h)
    create((8, 4, 6, 10), 1, 0)
    assert L.gbds_op_set_site_order(h, 2) == 5
    assert L.gbds_op_set_site_order(h, 0) == 0 and L.gbds_op_set_site_order(h, -1) == 0 and order() == 0
    L.gbds_op_destroy(h)
    # 32^3x64, 16 rhs, FP32 pairs, recon 12: 512-site planes of 16 * 192 + 8 * 48 bytes a site
    create((32, 32, 32, 64), 16, 3, recon=12)
    assert order() == 16
    L.gbds_op_destroy(h)
    for nrhs, fmt, want in ((16, 3, 0), (32, 3, 12), (32, 0, 12), (32, 1, 0), (8, 0, 0)):
        create((24, 24, 24, 48), nrhs, fmt)
        assert order() == want, (nrhs, fmt)
        L.gbds_op_destroy(h)
    # a z extent beyond the slab field's 16 bits: 2-site planes of 32 rhs
    # (6528 B a site) fit 2451 planes in the budget -> 2048, the largest
    # divisor of 65536 below that; a slab of 32768 planes is refused
    create((2, 2, 65536, 2), 32, 3)
    assert order() == 2048
    assert L.gbds_op_set_site_order(h, 32768) == 5 and order() == 2048
    assert L.gbds_op_set_site_order(h, 65536) == 0 and order() == 0
    L.gbds_op_destroy(h)


def test_double_float_format_validation(libs):
    """GBDS_SPINOR_DOUBLE_FLOAT (4): prec 64 and one rhs, 3D or 4D; fields of
    the FP64 size; the FP64 register-cap variants; no site order."""
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    h = ctypes.c_void_p()
    d = (ctypes.c_int * 4)(4, 4, 4, 6)
    assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 32, 18, 1, 4) == 5
    assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 64, 18, 2, 4) == 5
    assert L.gbds_op_create_ex(ctypes.byref(h), d, 4, 64, 18, 1, 5) == 1
    for nd in (4, 3):
        assert L.gbds_op_create_ex(ctypes.byref(h), d, nd, 64, 12, 1, 4) == 0
        ref = ctypes.c_void_p()
        assert L.gbds_op_create_ex(ctypes.byref(ref), d, nd, 64, 12, 1, 0) == 0
        assert L.gbds_op_spinor_bytes(h) == L.gbds_op_spinor_bytes(ref)
        assert L.gbds_op_gauge_bytes(h) == L.gbds_op_gauge_bytes(ref)
        assert L.gbds_op_num_variants(h) == L.gbds_op_num_variants(ref) == 3
        assert L.gbds_op_set_site_order(h, 2) == 5
        L.gbds_op_destroy(ref)
        L.gbds_op_destroy(h)

