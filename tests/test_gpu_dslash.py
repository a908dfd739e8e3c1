"""Parity of the GPU Dslash with the reference (golden vectors) and the
oracle, through the C ABI.  Tolerances, per site ||got - ref|| / ||ref||:
1e-6 for FP32 and 1e-13 for FP64."""
import numpy as np
import pytest

import oracle as O
from golden_data import SITE_TOL, check_against_golden, layout, load

pytestmark = pytest.mark.gpu

MAN, ARR = load()
CASES = sorted(MAN["cases"])


@pytest.fixture(scope="module")
def dropin():
    import __graft_entry__ as g
    g.build()
    from sse_wilson_dslash_gb300 import legacy
    legacy.set_exit_on_error(False)
    return {32: legacy.SSEDslash(32), 64: legacy.SSEDslash(64)}


def _init(d, nd, dims, kind, lol):
    O.set_callback_layout(kind, dims, lol if kind == O.LAYOUT_PERM else None)
    gc, gl, nn = O.callbacks()
    (d.init_sse_su3dslash if nd == 4 else d.init_sse_su3dslash_3d)(dims, gc, gl, nn)


def _free(d, nd):
    (d.free_sse_su3dslash if nd == 4 else d.free_sse_su3dslash_3d)()


def _apply(d, nd, u, psi, res, isign, cb):
    (d.sse_su3dslash_wilson if nd == 4 else d.sse_su3dslash_wilson_3d)(u, psi, res, isign, cb)


@pytest.mark.parametrize("recon,access", [(18, 0), (18, 1), (12, 0)])
@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("name", CASES)
def test_dropin_matches_reference_golden(dropin, name, prec, recon, access):
    """access 0: kernels read/write the host arrays directly where the GPU can
    reach them; 1: staged through cudaMemcpyAsync."""
    from sse_wilson_dslash_gb300 import legacy
    c = MAN["cases"][name]
    dims, nd = tuple(c["dims"]), c["nd"]
    kind, lol = layout(c, dims)
    d = dropin[prec]
    legacy.set_recon(recon)
    legacy.set_host_access(access)
    try:
        _init(d, nd, dims, kind, lol)
        u, psi = O.make_inputs(dims, MAN["seeds"]["gauge"], MAN["seeds"]["spinor"], c["gauge"])
        u, psi = u.astype(d.dtype), psi.astype(d.dtype)
        V = O.volume(dims)
        for isign in (1, -1):
            for cb in (0, 1):
                res = np.full((V, 4, 3, 2), 3.25, d.dtype)
                _apply(d, nd, u, psi, res, isign, cb)
                other = O.target_sites(nd, dims, lol, 1 - cb)  # sites of parity cb
                assert np.all(res.reshape(V, 24)[other] == 3.25), "wrote the source checkerboard"
                res.reshape(V, 24)[other] = 0.0
                check_against_golden(MAN, ARR, name, prec, isign, cb, res)
                ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
                assert O.site_rel_err(res, ref, O.target_sites(nd, dims, lol, cb)) <= SITE_TOL[prec]
        if access == 1 or kind == O.LAYOUT_PERM or kind == O.LAYOUT_LEX:
            assert legacy.last_path() == 0
    finally:
        _free(d, nd)
        legacy.set_recon(18)
        legacy.set_host_access(0)


def test_refcount_keeps_first_lattice(dropin):
    from sse_wilson_dslash_gb300 import legacy
    d = dropin[32]
    dims = (4, 4, 4, 4)
    _init(d, 4, dims, O.LAYOUT_CB2, None)
    _init(d, 4, (8, 8, 8, 8), O.LAYOUT_CB2, None)  # refcount 2, lattice unchanged
    assert legacy.refcount(32, 4) == 2
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, psi = O.make_inputs(dims)
    u, psi = u.astype(np.float32), psi.astype(np.float32)
    res = np.zeros((256, 4, 3, 2), np.float32)
    _free(d, 4)
    assert legacy.refcount(32, 4) == 1
    _apply(d, 4, u, psi, res, 1, 1)
    ref = O.dslash_plain(4, dims, lol, u, psi, 1, 1)
    assert O.site_rel_err(res, ref, O.target_sites(4, dims, lol, 1)) <= 1e-6
    _free(d, 4)
    assert legacy.refcount(32, 4) == 0


def test_bad_isign_is_noop_and_python_callbacks(dropin):
    d = dropin[64]
    dims = (2, 2, 2, 4)
    lex = lambda c: c[0] + 2 * (c[1] + 2 * (c[2] + 2 * c[3]))  # noqa: E731

    def coords(c, node, lin):
        c[0], c[1], c[2], c[3] = lin % 2, (lin // 2) % 2, (lin // 4) % 2, lin // 8

    d.init_sse_su3dslash(dims, coords, lex, None)
    try:
        u, psi = O.make_inputs(dims)
        res = np.full((32, 4, 3, 2), 9.0)
        for isign in (0, 2, -2):
            _apply(d, 4, u, psi, res, isign, 0)
        assert np.all(res == 9.0)
        lol = O.layout_table(O.LAYOUT_LEX, dims)
        _apply(d, 4, u, psi, res, -1, 0)
        ref = O.dslash_plain(4, dims, lol, u, psi, -1, 0, res=np.full((32, 4, 3, 2), 9.0))
        assert np.max(np.abs(res - ref)) < 1e-12
    finally:
        _free(d, 4)


@pytest.mark.parametrize("nd,dims", [(4, (2, 2, 2, 2)), (4, (2, 6, 2, 4)), (3, (2, 2, 2, 1)),
                                     (3, (6, 2, 4, 3)), (4, (16, 8, 4, 2))])
@pytest.mark.parametrize("prec", [32, 64])
def test_edge_lattices(dropin, nd, dims, prec):
    d = dropin[prec]
    kind = O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D
    lol = O.layout_table(kind, dims)
    _init(d, nd, dims, kind, None)
    try:
        u, psi = O.make_inputs(dims, 11, 12)
        u, psi = u.astype(d.dtype), psi.astype(d.dtype)
        V = O.volume(dims)
        for isign in (1, -1):
            for cb in (0, 1):
                res = np.zeros((V, 4, 3, 2), d.dtype)
                _apply(d, nd, u, psi, res, isign, cb)
                ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
                assert O.site_rel_err(res, ref, O.target_sites(nd, dims, lol, cb)) <= SITE_TOL[prec]
    finally:
        _free(d, nd)


def test_pinned_host_arrays_take_the_direct_path(dropin):
    """Pinned host arrays are read and written in place by the layout kernels."""
    import torch
    from sse_wilson_dslash_gb300 import legacy
    d = dropin[32]
    dims = (8, 4, 4, 8)
    _init(d, 4, dims, O.LAYOUT_CB2, None)
    try:
        u, psi = O.make_inputs(dims, 31, 32)
        V = O.volume(dims)
        ut = torch.from_numpy(u.astype(np.float32).ravel()).pin_memory()
        pt = torch.from_numpy(psi.astype(np.float32).ravel()).pin_memory()
        rt = torch.full((V * 24,), 2.5, dtype=torch.float32).pin_memory()
        legacy.set_gauge_cache(True)
        lol = O.layout_table(O.LAYOUT_CB2, dims)
        for isign, cb in ((1, 0), (-1, 1), (1, 1)):
            d.sse_su3dslash_wilson(ut, pt, rt, isign, cb)
            assert legacy.last_path() == 1
            res = rt.numpy().reshape(V, 4, 3, 2).copy()
            ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), psi.astype(np.float32), isign, cb)
            assert O.site_rel_err(res, ref, O.target_sites(4, dims, lol, cb)) <= 1e-6
        # gauge cache: a changed field behind the same pointer is only seen after invalidation
        ut.mul_(-1.0)
        legacy.invalidate_gauge()
        d.sse_su3dslash_wilson(ut, pt, rt, 1, 0)
        ref = O.dslash_plain(4, dims, lol, -u.astype(np.float32), psi.astype(np.float32), 1, 0)
        assert O.site_rel_err(rt.numpy().reshape(V, 4, 3, 2), ref, O.target_sites(4, dims, lol, 0)) <= 1e-6
    finally:
        legacy.set_gauge_cache(False)
        _free(d, 4)


def test_autotune_picks_a_valid_configuration_and_keeps_results():
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (16, 8, 8, 8)
    op = DslashOperator(dims, nd=4, prec=32, recon=18)
    g = torch.Generator(device="cuda").manual_seed(3)
    u = torch.randn(op.volume * 72, device="cuda", generator=g)
    psi = torch.randn(op.volume * 24, device="cuda", generator=g)
    gauge = op.pack_gauge(u)
    src = op.pack_spinor(psi, 0)
    before = op.apply(gauge, src, 1, 0).clone()
    block, variant = op.autotune(gauge, src, op.new_spinor())
    assert block % 32 == 0 and 0 <= variant < op.num_variants
    after = op.apply(gauge, src, 1, 0)
    torch.cuda.synchronize()
    assert torch.equal(before, after)
    op2 = DslashOperator(dims, nd=4, prec=32, recon=18)
    assert op2.autotune(gauge, src, op.new_spinor()) == (block, variant)  # cached per shape


# ---------------------------------------------------------------------------
# Device-resident operator (gbds_op_*)
# ---------------------------------------------------------------------------

def _device_fields(op, u, psi, torch):
    ud = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    pd = torch.from_numpy(np.ascontiguousarray(psi)).cuda()
    return op.pack_gauge(ud), pd


@pytest.mark.parametrize("recon", [18, 12])
@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("nd,dims,layout_kind", [(4, (8, 4, 6, 4), "canonical"), (3, (4, 6, 4, 5), "canonical"),
                                                  (4, (4, 4, 2, 6), "scrambled"), (3, (4, 2, 4, 3), "scrambled")])
def test_device_operator(nd, dims, layout_kind, prec, recon):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=nd, prec=prec, recon=recon)
    V = op.volume
    if layout_kind == "canonical":
        lol = O.layout_table(O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D, dims)
    else:
        lol = O.scrambled_table(dims, 3)
        # internal site i has coordinates internal_coords(i); its caller index:
        from sse_wilson_dslash_gb300.layouts import internal_coords
        x, y, z, t = internal_coords(dims, nd)
        lex = x + dims[0] * (y + dims[1] * (z + dims[2] * t))
        op.set_layout(lol[lex])
        assert not op.canonical
    dt = np.float32 if prec == 32 else np.float64
    u, psi = O.make_inputs(dims, 21, 22)
    u, psi = u.astype(dt), psi.astype(dt)
    gauge, pd = _device_fields(op, u, psi, torch)
    for isign in (1, -1):
        for cb in (0, 1):
            src = op.pack_spinor(pd, cb)
            out = op.apply(gauge, src, isign, cb)
            res = torch.zeros(V * 24, dtype=op.real_dtype, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            torch.cuda.synchronize()
            ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
            got = res.cpu().numpy()
            assert O.site_rel_err(got, ref, O.target_sites(nd, dims, lol, cb)) <= SITE_TOL[prec]
    op.close()


@pytest.mark.slow
@pytest.mark.parametrize("prec", [32, 64])
def test_production_lattice_properties(prec):
    """32^3x64: (a) every output site against the C oracle,
    (b) linearity, (c) <chi, D psi> = <D^dagger chi, psi> between checkerboards."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (32, 32, 32, 64)
    op = DslashOperator(dims, nd=4, prec=prec, recon=18)
    dt = torch.float32 if prec == 32 else torch.float64
    g = torch.Generator(device="cuda").manual_seed(5)
    V = op.volume
    # random links: any complex 3x3 is fine for linearity/adjointness
    u = torch.randn(V * 72, dtype=dt, device="cuda", generator=g)
    psi = torch.randn(V * 24, dtype=dt, device="cuda", generator=g)
    phi = torch.randn(V * 24, dtype=dt, device="cuda", generator=g)
    gauge = op.pack_gauge(u)
    full = torch.zeros(V * 24, dtype=dt, device="cuda")

    def D(field, isign, cb):
        s = op.pack_spinor(field, cb)
        o = op.apply(gauge, s, isign, cb)
        out = torch.zeros(V * 24, dtype=dt, device="cuda")
        op.unpack_spinor(o, 1 - cb, out)
        return out.double()

    a, b = 0.75, -1.5
    lhs = D(a * psi + b * phi, 1, 0)
    rhs = a * D(psi, 1, 0) + b * D(phi, 1, 0)
    tol = 1e-5 if prec == 32 else 1e-12
    assert (lhs - rhs).norm() / rhs.norm() < tol
    # adjointness: chi on parity 1 (target of cb=0), psi on parity 0
    Dpsi = D(psi, 1, 0)          # parity 1
    Ddag_chi = D(phi, -1, 1)     # parity 0
    Vh = V // 2
    c1 = phi.double().view(V, 24)[Vh:].reshape(-1)
    p0 = psi.double().view(V, 24)[:Vh].reshape(-1)
    lhs_ip = torch.dot(c1, Dpsi.view(V, 24)[Vh:].reshape(-1))
    rhs_ip = torch.dot(Ddag_chi.view(V, 24)[:Vh].reshape(-1), p0)
    # real parts of <chi, D psi> and <D^dag chi, psi> agree (the imaginary
    # parts follow from the same identity for i*chi)
    assert abs(lhs_ip - rhs_ip) / abs(lhs_ip) < (1e-4 if prec == 32 else 1e-11)
    # every site against the C oracle (FP64, OpenMP)
    uu = u.cpu().numpy().reshape(V, 4, 3, 3, 2)
    pp = psi.cpu().numpy().reshape(V, 4, 3, 2)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    ref = O.dslash_plain(4, dims, lol, uu, pp, 1, 0)
    got = Dpsi.cpu().numpy()
    ts = O.target_sites(4, dims, lol, 0)
    assert O.site_rel_err(got, ref, ts) <= SITE_TOL[prec]
    del full
    op.close()
