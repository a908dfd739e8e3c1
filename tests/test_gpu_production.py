"""Parity at the production sizes the benchmark runs (GPU): every target site
of the GPU operator against the C oracle (orc_dslash_plain, FP64, OpenMP) on
the same inputs, per site ||got - ref|| / ||ref|| <= 1e-6 (FP32) and 1e-13
(FP64).

* 4D 32^3x64: FP32 and FP64, links with 18 and 12 reals, isign +1/-1, cb 0/1
  (the reference's operator, lib/sse_su3dslash_32bit_scalar.c:159-180 and
  lib/sse_su3dslash_64bit_scalar.c:150-170);
* 3D 24^3x48 in the cb3d site order: the same combinations
  (lib/sse_su3dslash_32bit_scalar_3d.c:150-359);
* the FP64 operator in double-float arithmetic (GBDS_SPINOR_DOUBLE_FLOAT) on
  both, at the FP64 tolerance;
* the drop-in C ABI (sse_su3dslash_wilson of libgbdslash32.so / 64.so) on
  32^3x64 with the QDP++ cb2 callbacks, kernels reading the host arrays in
  place and staged through copies; the source checkerboard of res is left
  untouched.

Inputs: random SU(3) links (Gaussian rows, Gram-Schmidt, row 2 = conj(row 0 x
row 1)) and N(0,1) spinors, generated on the device and rounded to the
operator's precision before the oracle sees them.
"""
import numpy as np
import pytest

import oracle as O
from golden_data import SITE_TOL

pytestmark = pytest.mark.gpu

DIMS_4D = (32, 32, 32, 64)
DIMS_3D = (24, 24, 24, 48)
COMBOS = [(1, 0), (1, 1), (-1, 0), (-1, 1)]


def _inputs(dims, prec, seed):
    """Packed (u, psi) as numpy arrays of the operator's real type."""
    import torch
    from bench import su3_links
    V = O.volume(dims)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    dt = torch.float32 if prec == 32 else torch.float64
    u = su3_links(V * 4, gen, torch).to(dt).reshape(V, 4, 3, 3, 2)
    psi = torch.randn(V, 4, 3, 2, dtype=dt, device="cuda", generator=gen)
    return u.cpu().numpy(), psi.cpu().numpy()


def _device_operator_check(nd, dims, prec, recon, seed, fmt="native"):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=nd, prec=prec, recon=recon, spinor_format=fmt)
    assert op.canonical
    u, psi = _inputs(dims, prec, seed)
    V = op.volume
    lol = O.layout_table(O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D, dims)
    gauge = op.pack_gauge(torch.from_numpy(u.ravel()).cuda())
    pd = torch.from_numpy(psi.ravel()).cuda()
    errs = {}
    for isign, cb in COMBOS:
        out = op.apply(gauge, op.pack_spinor(pd, cb), isign, cb)
        res = torch.zeros(V * 24, dtype=op.real_dtype, device="cuda")
        op.unpack_spinor(out, 1 - cb, res)
        got = res.cpu().numpy()
        ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
        ts = O.target_sites(nd, dims, lol, cb)
        errs[(isign, cb)] = O.site_rel_err(got, ref, ts)
        # the source checkerboard of the unpacked array stays untouched
        assert not np.any(got.reshape(V, 24)[O.target_sites(nd, dims, lol, 1 - cb)])
    op.close()
    for k, e in errs.items():
        assert e <= SITE_TOL[prec], (nd, dims, prec, recon, fmt, k, e)
    return errs


@pytest.mark.parametrize("recon", [18, 12])
@pytest.mark.parametrize("prec", [32, 64])
def test_4d_32x32x32x64_every_site_every_combination(prec, recon):
    _device_operator_check(4, DIMS_4D, prec, recon, seed=40 + prec + recon)


@pytest.mark.parametrize("nd,dims", [(4, DIMS_4D), (3, DIMS_3D)])
@pytest.mark.parametrize("recon", [18, 12])
def test_double_float_at_production_size(nd, dims, recon):
    """The FP64 operator in double-float arithmetic (GBDS_SPINOR_DOUBLE_FLOAT)
    at the production sizes, every target site and combination against the
    oracle at the FP64 tolerance (1e-13)."""
    _device_operator_check(nd, dims, 64, recon, seed=70 + nd + recon, fmt="double_float")


@pytest.mark.parametrize("recon", [18, 12])
@pytest.mark.parametrize("prec", [32, 64])
def test_3d_24x24x24x48_every_site_every_combination(prec, recon):
    _device_operator_check(3, DIMS_3D, prec, recon, seed=50 + prec + recon)


@pytest.mark.parametrize("access", [0, 1])
@pytest.mark.parametrize("prec", [32, 64])
def test_dropin_abi_32x32x32x64(prec, access):
    """sse_su3dslash_wilson on host arrays with the oracle's QDP++ cb2
    callbacks: access 0 lets the layout kernels read u/psi and write res in
    place, access 1 stages every array through cudaMemcpyAsync."""
    from sse_wilson_dslash_gb300 import legacy
    legacy.set_exit_on_error(False)
    legacy.set_host_access(access)
    d = legacy.SSEDslash(prec)
    dims = DIMS_4D
    O.set_callback_layout(O.LAYOUT_CB2, dims)
    d.init_sse_su3dslash(dims, *O.callbacks())
    try:
        u, psi = _inputs(dims, prec, seed=60 + prec)
        V = O.volume(dims)
        lol = O.layout_table(O.LAYOUT_CB2, dims)
        for isign, cb in COMBOS if prec == 32 else COMBOS[:2]:
            res = np.full((V, 4, 3, 2), 7.5, d.dtype)
            d.sse_su3dslash_wilson(u, psi, res, isign, cb)
            src = O.target_sites(4, dims, lol, 1 - cb)
            assert np.all(res.reshape(V, 24)[src] == 7.5), "wrote the source checkerboard"
            ref = O.dslash_plain(4, dims, lol, u, psi, isign, cb)
            err = O.site_rel_err(res, ref, O.target_sites(4, dims, lol, cb))
            assert err <= SITE_TOL[prec], (prec, access, isign, cb, err)
        if access == 1:
            assert legacy.last_path() == 0
    finally:
        d.free_sse_su3dslash()
        legacy.set_host_access(0)


@pytest.mark.parametrize("prec", [32, 64])
def test_dropin_abi_3d_24x24x24x48(prec):
    """sse_su3dslash_wilson_3d with the cb3d callbacks (t fastest)."""
    from sse_wilson_dslash_gb300 import legacy
    legacy.set_exit_on_error(False)
    d = legacy.SSEDslash(prec)
    dims = DIMS_3D
    O.set_callback_layout(O.LAYOUT_CB3D, dims)
    d.init_sse_su3dslash_3d(dims, *O.callbacks())
    try:
        u, psi = _inputs(dims, prec, seed=70 + prec)
        V = O.volume(dims)
        lol = O.layout_table(O.LAYOUT_CB3D, dims)
        for isign, cb in ((1, 0), (-1, 1)):
            res = np.zeros((V, 4, 3, 2), d.dtype)
            d.sse_su3dslash_wilson_3d(u, psi, res, isign, cb)
            ref = O.dslash_plain(3, dims, lol, u, psi, isign, cb)
            err = O.site_rel_err(res, ref, O.target_sites(3, dims, lol, cb))
            assert err <= SITE_TOL[prec], (prec, isign, cb, err)
    finally:
        d.free_sse_su3dslash_3d()
