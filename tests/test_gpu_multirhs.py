"""Several right-hand sides per site and 16-bit spinor storage (GPU), each
right-hand side checked against the oracle."""
import numpy as np
import pytest

import oracle as O
from formats import TOL, TOL_TC, site_err, stored

pytestmark = pytest.mark.gpu

def _round(psi, fmt):
    return stored(psi, fmt)


@pytest.mark.parametrize("fmt", ["native", "f32_pairs", "bf16", "f16"])
@pytest.mark.parametrize("nrhs", [1, 2, 4, 8, 16, 32])
def test_multi_rhs_matches_oracle(nrhs, fmt):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    if fmt != "native" and nrhs in (2, 16):
        pytest.skip("covered by the other counts")
    dims = (8, 4, 6, 4)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    for recon in (18, 12):
        op = DslashOperator(dims, nd=4, prec=32, recon=recon, nrhs=nrhs, spinor_format=fmt)
        gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
        packed = torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda()
        for isign, cb in ((1, 0), (-1, 1)):
            src = op.pack_spinor(packed, cb)
            out = op.apply(gauge, src, isign, cb)
            res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            got = res.cpu().numpy().reshape(nrhs, V, 24)
            ts = O.target_sites(4, dims, lol, cb)
            for r in range(nrhs):
                ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb)
                err = O.site_rel_err(got[r], ref, ts)
                assert err <= TOL[fmt], (recon, isign, cb, r, err)
        op.close()


def test_multi_rhs_bytes_accounting():
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator((4, 4, 4, 4), nrhs=16, spinor_format="bf16", recon=12)
    assert op.bytes_per_site == 2 * 48 + 8 * 48 / 16
    assert op.spinor_bytes == 48 * op.stride * 16
    op.close()


@pytest.mark.parametrize("fmt", ["native", "f32_pairs"])
def test_fp32_field_layouts_match_the_header(fmt):
    """The packed bytes of the two FP32 multi-rhs formats are the layouts
    include/gbdslash.h documents: element (k, h, r) at
    k*stride*nrhs + h*nrhs + r, 16-byte component k holding complex elements
    2k and 2k+1 (FP32), or (s0c.r, s1c.r, s0c.i, s1c.i) for k = c < 3 and
    (s2c.r, s3c.r, s2c.i, s3c.i) for k = 3 + c (FP32 spin pairs)."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims, nrhs = (4, 4, 4, 4), 2
    op = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
    V, Vh, stride = op.volume, op.volume_cb, op.stride
    # value = r * 100000 + site * 100 + spin * 10 + colour * 2 + reim: exact in FP32
    r_, site, spin, col, ri = np.meshgrid(np.arange(nrhs), np.arange(V), np.arange(4), np.arange(3), np.arange(2),
                                          indexing="ij")
    psi = (r_ * 100000 + site * 100 + spin * 10 + col * 2 + ri).astype(np.float32)
    for parity in (0, 1):
        raw = op.pack_spinor(torch.from_numpy(psi.ravel()).cuda(), parity)
        got = raw.view(torch.float32).cpu().numpy().reshape(6, stride, nrhs, 4)[:, :Vh]
        s = psi[:, parity * Vh:(parity + 1) * Vh].transpose(1, 0, 2, 3, 4)  # [h][r][spin][colour][reim]
        want = np.empty((6, Vh, nrhs, 4), dtype=np.float32)
        for k in range(6):
            if fmt == "native":
                e0, e1 = 2 * k, 2 * k + 1
                want[k] = np.stack([s[:, :, e0 // 3, e0 % 3, 0], s[:, :, e0 // 3, e0 % 3, 1],
                                    s[:, :, e1 // 3, e1 % 3, 0], s[:, :, e1 // 3, e1 % 3, 1]], axis=-1)
            else:
                a, c = (0, k) if k < 3 else (2, k - 3)
                want[k] = np.stack([s[:, :, a, c, 0], s[:, :, a + 1, c, 0], s[:, :, a, c, 1], s[:, :, a + 1, c, 1]],
                                   axis=-1)
        np.testing.assert_array_equal(got, want)
    op.close()


# Tensor-core form: besides the storage rounding above, the projected half
# spinor and the link enter the MMA rounded to the 16-bit operand type (one
# more rounding of each, FP32 accumulation), well inside the same per-site
# bounds.
# (8, 4, 6, 4): one tile per CTA; (16, 8, 8, 16): every persistent CTA walks
# several tiles, so the loads of the next tile overlap the last MMA of this one.
@pytest.mark.parametrize("dims", [(8, 4, 6, 4), (16, 8, 8, 16)])
@pytest.mark.parametrize("fmt", ["bf16", "f16"])
@pytest.mark.parametrize("nrhs", [16, 32])
def test_tensor_core_multi_rhs_matches_oracle(nrhs, fmt, dims):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(100 + nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    for recon in ((18, 12) if V < 4096 else (18,)):
        op = DslashOperator(dims, nd=4, prec=32, recon=recon, nrhs=nrhs, spinor_format=fmt)
        op.set_tensor_cores(True)
        gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
        packed = torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda()
        for isign, cb in ((1, 0), (-1, 1), (1, 1), (-1, 0)):
            src = op.pack_spinor(packed, cb)
            out = op.apply(gauge, src, isign, cb)
            op.check()
            res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            got = res.cpu().numpy().reshape(nrhs, V, 24)
            ts = O.target_sites(4, dims, lol, cb)
            for r in range(nrhs):
                ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb)
                err = O.site_rel_err(got[r], ref, ts)
                assert err <= TOL_TC[fmt], (recon, isign, cb, r, err)
        op.close()


def test_tensor_cores_need_16bit_and_16_or_32_rhs():
    from sse_wilson_dslash_gb300.device import DslashOperator
    from sse_wilson_dslash_gb300 import _lib
    for nrhs, fmt in ((32, "native"), (32, "f32_pairs"), (8, "bf16"), (1, "f16")):
        op = DslashOperator((4, 4, 4, 4), nrhs=nrhs, spinor_format=fmt)
        with pytest.raises(_lib.GbdsError):
            op.set_tensor_cores(True)
        op.close()


@pytest.mark.parametrize("fmt", ["bf16", "f16", "f32_pairs"])
def test_autotune_chooses_between_cuda_and_tensor_cores(fmt):
    """The autotuner times the CUDA-core variants (and, for 16-bit storage,
    the tensor-core kernel) for a 32-rhs operator, then for a CUDA-core pick
    the site order (natural, or z slabs of Lz/8 planes and up: here 0, 2 or
    4); the pick (cached) gives the same answer as the oracle, and a second
    operator of the same shape takes the cached site order."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims, nrhs = (8, 8, 8, 8), 32
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(9)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    op = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
    gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
    src = op.pack_spinor(torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda(), 0)
    op.autotune(gauge, src, op.new_spinor())
    assert op.site_order() in (0, 2, 4)
    out = op.apply(gauge, src, 1, 0)
    op.check()
    res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
    op.unpack_spinor(out, 1, res)
    got = res.cpu().numpy().reshape(nrhs, V, 24)
    ts = O.target_sites(4, dims, lol, 0)
    for r in range(0, nrhs, 7):
        ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), 1, 0)
        assert O.site_rel_err(got[r], ref, ts) <= TOL_TC.get(fmt, TOL[fmt])
    again = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
    again.autotune(gauge, src, again.new_spinor())  # from the cache
    assert again.tuning() == op.tuning() and again.site_order() == op.site_order()
    again.close()
    op.close()


# Smallest and uneven shapes for the tensor-core kernel: a 2^4 lattice (two
# tiles with 32 rhs), Lx = 2 (half extent 1: the division-free path of the
# coordinate decomposition) and extents of different lengths in every
# direction.
@pytest.mark.parametrize("dims", [(2, 2, 2, 2), (2, 4, 6, 2), (6, 2, 4, 10)])
@pytest.mark.parametrize("nrhs", [16, 32])
def test_tensor_core_edge_lattices(dims, nrhs):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    fmt = "bf16"
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(sum(dims) + nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    op = DslashOperator(dims, nd=4, prec=32, recon=12, nrhs=nrhs, spinor_format=fmt)
    op.set_tensor_cores(True)
    gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
    packed = torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda()
    for isign, cb in ((1, 1), (-1, 0)):
        out = op.apply(gauge, op.pack_spinor(packed, cb), isign, cb)
        op.check()
        res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
        op.unpack_spinor(out, 1 - cb, res)
        got = res.cpu().numpy().reshape(nrhs, V, 24)
        ts = O.target_sites(4, dims, lol, cb)
        for r in range(nrhs):
            ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb)
            assert O.site_rel_err(got[r], ref, ts) <= TOL_TC[fmt], (dims, isign, cb, r)
    op.close()


def test_tensor_core_wait_times_out_and_reports():
    """A bounded mbarrier wait on a barrier that nothing completes gives up,
    reports it, and leaves the context usable: a tensor-core Dslash runs
    correctly afterwards."""
    from sse_wilson_dslash_gb300 import _lib
    _lib.check(_lib.core().gbds_tc_wait_selftest(4096))
    test_tensor_core_edge_lattices((2, 4, 6, 2), 32)


# ---------------------------------------------------------------------------
# The configured size: 24^3x48, one random SU(3) field, up to 32 rhs
# ---------------------------------------------------------------------------

PROD_DIMS = (24, 24, 24, 48)
PROD_ISIGN, PROD_CB = -1, 0


@pytest.fixture(scope="module")
def production():
    """Inputs at 24^3x48 and the oracle's outputs for all 32 rhs, per stored
    format (FP32, bfloat16, half + norm), on the target sites, on the device."""
    import torch
    from bench import su3_links
    dims, nrhs = PROD_DIMS, 32
    V = O.volume(dims)
    gen = torch.Generator(device="cuda").manual_seed(2024)
    u = su3_links(V * 4, gen, torch).float().reshape(-1)
    psi = torch.randn(nrhs, V * 24, dtype=torch.float32, device="cuda", generator=gen)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    ts = O.target_sites(4, dims, lol, PROD_CB)
    uh, ph = u.cpu().numpy(), psi.cpu().numpy()
    refs = {}
    for kind in ("native", "bf16", "f16"):
        src = stored(ph, kind)
        refs[kind] = torch.from_numpy(np.stack([
            O.dslash_plain(4, dims, lol, uh, src[r], PROD_ISIGN, PROD_CB).reshape(V, 24)[ts]
            for r in range(nrhs)])).cuda()
    return dict(u=u, psi=psi, refs=refs, ts=torch.from_numpy(ts).cuda(), V=V)


def _production_error(production, nrhs, fmt, variant=None, tc=False, zblock=-1):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    P = production
    op = DslashOperator(PROD_DIMS, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
    if tc:
        op.set_tensor_cores(True)
    elif variant is not None:
        op.set_tuning(0, variant)
    op.set_site_order(zblock)
    gauge = op.pack_gauge(P["u"])
    out = op.apply(gauge, op.pack_spinor(P["psi"][:nrhs].reshape(-1), PROD_CB), PROD_ISIGN, PROD_CB)
    op.check()
    res = torch.zeros(nrhs * P["V"] * 24, dtype=torch.float32, device="cuda")
    op.unpack_spinor(out, 1 - PROD_CB, res)
    got = res.view(nrhs, P["V"], 24)[:, P["ts"]].double()
    ref = P["refs"]["native" if fmt == "f32_pairs" else fmt][:nrhs]
    op.close()
    return ((got - ref).norm(dim=2) / ref.norm(dim=2)).max().item()


@pytest.mark.slow
@pytest.mark.parametrize("fmt,variants", [("native", (0, 1, 2, 3)), ("f32_pairs", (1, 2, 3)), ("bf16", (0, 2, 3, 4)),
                                          ("f16", (2, 3, 4))])
@pytest.mark.parametrize("nrhs", [16, 32])
def test_multi_rhs_24x24x24x48_every_rhs_against_oracle(production, nrhs, fmt, variants):
    """Every rhs and target site at the configured size, for the CUDA-core
    variants the autotuner chooses among (0 plain, 1 packed colour multiply,
    2 fully packed), within the storage format's bound."""
    for v in variants:
        err = _production_error(production, nrhs, fmt, variant=v)
        assert err <= TOL[fmt], (nrhs, fmt, v, err)


@pytest.mark.slow
@pytest.mark.parametrize("fmt", ["bf16", "f16"])
@pytest.mark.parametrize("nrhs", [16, 32])
def test_tensor_core_24x24x24x48_every_rhs_against_oracle(production, nrhs, fmt):
    err = _production_error(production, nrhs, fmt, tc=True)
    assert err <= TOL_TC[fmt], (nrhs, fmt, err)


@pytest.mark.parametrize("fmt", ["native", "f32_pairs", "bf16", "f16"])
@pytest.mark.parametrize("nrhs", [8, 16, 32])
def test_packed_fp32x2_variant_matches_oracle(nrhs, fmt):
    """Variants 1 (links staged per CTA, colour multiply in packed FP32x2
    arithmetic) and 2 (the whole hop in packed FP32x2; 16-bit and FP32-pair
    storage) of the multi-RHS kernel against the oracle."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (8, 4, 6, 4)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(300 + nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    variants = (1, 2, 3, 4)
    for recon, variant in [(rc, v) for rc in (18, 12) for v in variants]:
        op = DslashOperator(dims, nd=4, prec=32, recon=recon, nrhs=nrhs, spinor_format=fmt)
        assert op.num_variants == 5
        op.set_tuning(0, variant)
        gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
        packed = torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda()
        for isign, cb in ((1, 0), (-1, 1)):
            out = op.apply(gauge, op.pack_spinor(packed, cb), isign, cb)
            res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            got = res.cpu().numpy().reshape(nrhs, V, 24)
            ts = O.target_sites(4, dims, lol, cb)
            for r in range(nrhs):
                ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb)
                assert O.site_rel_err(got[r], ref, ts) <= TOL[fmt], (recon, variant, isign, cb, r)
        op.close()


@pytest.mark.parametrize("fmt", ["bf16", "f16", "f32_pairs", "native"])
@pytest.mark.parametrize("nrhs", [8, 16, 32])
def test_packed_variants_partial_last_cta(nrhs, fmt):
    """6x2x2x10: 120 sites a checkerboard, not a multiple of the 4-32 sites a
    CTA of the fully packed variants holds, so the last CTA is partly idle;
    variants 2, 3 and 4 against the oracle on every rhs."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (6, 2, 2, 10)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(500 + nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    for variant in (2, 3, 4):
        op = DslashOperator(dims, nd=4, prec=32, recon=12, nrhs=nrhs, spinor_format=fmt)
        op.set_tuning(0, variant)
        gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
        packed = torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda()
        for isign, cb in ((1, 1), (-1, 0)):
            out = op.apply(gauge, op.pack_spinor(packed, cb), isign, cb)
            res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            got = res.cpu().numpy().reshape(nrhs, V, 24)
            ts = O.target_sites(4, dims, lol, cb)
            for r in range(nrhs):
                ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb)
                assert O.site_rel_err(got[r], ref, ts) <= TOL[fmt], (variant, isign, cb, r)
        op.close()


@pytest.mark.parametrize("fmt,nrhs", [("native", 4), ("native", 16), ("f32_pairs", 16), ("bf16", 32), ("f16", 8)])
def test_site_orders_match_oracle(fmt, nrhs):
    """The z-slab site orders of gbds_op_set_site_order against the natural
    order (bit-identical outputs: every site runs the same arithmetic in any
    order) and the oracle, for every CUDA-core variant: 6x2x6x10 has planes of
    6 sites, so CTAs straddle planes and slabs; slabs of 1, 2 and 3 planes."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (6, 2, 6, 10)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(700 + nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    isign, cb = -1, 1
    ts = O.target_sites(4, dims, lol, cb)
    refs = [O.dslash_plain(4, dims, lol, u.astype(np.float32), _round(psis[r], fmt), isign, cb) for r in range(nrhs)]
    variants = (0, 1, 2, 3, 4)
    for variant in variants:
        op = DslashOperator(dims, nd=4, prec=32, recon=12, nrhs=nrhs, spinor_format=fmt)
        op.set_tuning(0, variant)
        gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
        src = op.pack_spinor(torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda(), cb)
        op.set_site_order(0)
        assert op.site_order() == 0
        natural = op.new_spinor().zero_()
        op.apply(gauge, src, isign, cb, out=natural)
        for zb in (1, 2, 3):
            op.set_site_order(zb)
            assert op.site_order() == zb
            out = op.new_spinor().zero_()
            op.apply(gauge, src, isign, cb, out=out)
            torch.cuda.synchronize()
            assert torch.equal(out, natural), (variant, zb)
        res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
        op.unpack_spinor(natural, 1 - cb, res)
        got = res.cpu().numpy().reshape(nrhs, V, 24)
        for r in range(nrhs):
            assert O.site_rel_err(got[r], refs[r], ts) <= TOL[fmt], (variant, r)
        op.close()


@pytest.mark.slow
@pytest.mark.parametrize("fmt,nrhs,variant,zblock", [("bf16", 32, 4, 4), ("f16", 16, 3, 3), ("native", 32, 1, 2),
                                                     ("f32_pairs", 16, 2, 6)])
def test_site_order_24x24x24x48_every_rhs_against_oracle(production, fmt, nrhs, variant, zblock):
    """Slabs chosen by hand at the configured size, every rhs and target site
    against the oracle (the defaults' slabs are covered by the tests above)."""
    err = _production_error(production, nrhs, fmt, variant=variant, zblock=zblock)
    assert err <= TOL[fmt], (nrhs, fmt, variant, zblock, err)

