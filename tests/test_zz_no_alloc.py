"""gbds_dslash_packed_noalloc_f32: the packed-layout Dslash for callers that
cannot allocate device memory (a framework that owns all device memory
through its own pool, a fixed memory budget, or a loop that cannot take the
device-wide synchronisation of cudaFree).  Its scratch is a static 12 MiB
device array, so it takes lattices of at most 32768 sites.

Checked through the C ABI against the allocating operator-handle path
(gbds_op_pack_* + gbds_op_dslash + gbds_op_unpack_spinor) on the same inputs,
on two calls in a row, and against the CPU oracle, with the per-site
tolerance of the FP32 parity tests; the device's free memory is the same
before and after a call.  This file is collected last."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

MAX_SITES = 32768
FP32_SITE_TOL = 1e-6


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    from sse_wilson_dslash_gb300 import _lib
    L = _lib.core()
    L.gbds_dslash_packed_noalloc_f32.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_void_p]
    return L


def _fields(torch, V, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    u = torch.randn(V * 72, dtype=torch.float32, device="cuda", generator=g)
    psi = torch.randn(V * 24, dtype=torch.float32, device="cuda", generator=g)
    return u, psi


def _allocating(dims, nd, u, psi, isign, cb, torch):
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=nd, prec=32, recon=18)
    out = torch.zeros(op.volume * 24, dtype=torch.float32, device="cuda")
    gauge = op.pack_gauge(u)
    res = op.apply(gauge, op.pack_spinor(psi, cb), isign, cb)
    op.unpack_spinor(res, 1 - cb, out)
    torch.cuda.synchronize()
    op.close()
    return out


def _noalloc(lib, dims, nd, u, psi, isign, cb, torch, fill=0.0):
    out = torch.full((len(psi),), fill, dtype=torch.float32, device="cuda")
    d = (ctypes.c_int * 4)(*dims)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.gbds_dslash_packed_noalloc_f32(d, nd, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(psi.data_ptr()),
                                            ctypes.c_void_p(out.data_ptr()), isign, cb, s)
    assert rc == 0, lib.gbds_get_last_error()
    torch.cuda.synchronize()
    return out


def _site_err(got, ref, nd, dims, cb):
    from sse_wilson_dslash_gb300.layouts import internal_coords
    V = int(np.prod(dims))
    g = got.double().cpu().numpy().reshape(V, 24)
    r = ref.double().cpu().numpy().reshape(V, 24)
    x, y, z, t = internal_coords(dims, nd)  # canonical order: caller index == internal index
    par = (x + y + z + (t if nd == 4 else 0)) & 1
    tgt = np.nonzero(par == 1 - cb)[0]
    err = np.linalg.norm(g[tgt] - r[tgt], axis=1) / np.linalg.norm(r[tgt], axis=1)
    return float(err.max()), g, tgt


@pytest.mark.parametrize("nd,dims", [(4, (8, 8, 8, 8)), (4, (8, 8, 8, 64)), (3, (4, 6, 4, 5))])
def test_noalloc_matches_allocating_path_two_calls(lib, nd, dims):
    import torch
    V = int(np.prod(dims))
    assert V <= MAX_SITES
    for call, (seed, isign, cb) in enumerate([(1, 1, 0), (2, -1, 1)]):
        u, psi = _fields(torch, V, seed)
        ref = _allocating(dims, nd, u, psi, isign, cb, torch)
        got = _noalloc(lib, dims, nd, u, psi, isign, cb, torch, fill=5.0)
        err, g, tgt = _site_err(got, ref, nd, dims, cb)
        assert err <= FP32_SITE_TOL, (call, err)
        other = np.setdiff1d(np.arange(V), tgt)
        assert np.all(g[other] == 5.0), "wrote the source checkerboard"


def test_noalloc_rejects_lattices_above_the_limit(lib):
    import torch
    dims = (8, 8, 8, 66)  # 33792 sites > 32768
    u = torch.zeros(8, dtype=torch.float32, device="cuda")
    d = (ctypes.c_int * 4)(*dims)
    rc = lib.gbds_dslash_packed_noalloc_f32(d, 4, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(u.data_ptr()),
                                            ctypes.c_void_p(u.data_ptr()), 1, 0, None)
    assert rc == 1
    assert b"no-allocation limit of 32768 sites" in lib.gbds_get_last_error()


@pytest.mark.parametrize("nd,dims", [(4, (8, 8, 4, 8)), (3, (4, 6, 4, 5))])
def test_noalloc_matches_oracle(lib, nd, dims):
    """Seeded random SU(3) links and N(0,1) spinors in the QDP++ order (cb2 for
    4D, cb3d for 3D), every target site against the oracle, all four isign /
    cb combinations."""
    import torch
    V = int(np.prod(dims))
    lol = O.layout_table(O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D, dims)
    u, psi = O.make_inputs(dims, 101, 102)
    u, psi = u.astype(np.float32), psi.astype(np.float32)
    ud = torch.from_numpy(u.ravel()).cuda()
    pd = torch.from_numpy(psi.ravel()).cuda()
    for isign, cb in ((1, 0), (1, 1), (-1, 0), (-1, 1)):
        got = _noalloc(lib, dims, nd, ud, pd, isign, cb, torch).cpu().numpy()
        ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
        assert O.site_rel_err(got, ref, O.target_sites(nd, dims, lol, cb)) <= FP32_SITE_TOL, (isign, cb)


def test_noalloc_leaves_device_free_memory_unchanged(lib):
    """After a first call (which may load the library's device code and with
    it the static array), a further call changes the device's free memory by
    nothing: it allocates no device memory."""
    import torch
    dims = (8, 8, 8, 16)
    V = int(np.prod(dims))
    u, psi = _fields(torch, V, 7)
    out = torch.zeros(V * 24, dtype=torch.float32, device="cuda")
    d = (ctypes.c_int * 4)(*dims)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (d, 4, ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(out.data_ptr()))
    assert lib.gbds_dslash_packed_noalloc_f32(*args, 1, 0, s) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for isign, cb in ((-1, 1), (1, 0)):
        assert lib.gbds_dslash_packed_noalloc_f32(*args, isign, cb, s) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
