"""The double-float FP64 operator (GPU, GBDS_SPINOR_DOUBLE_FLOAT): FP64
fields held as hi + lo FP32 pairs and computed on the FP32 pipes, against the
oracle's FP64 Dslash at the FP64 per-site tolerance,
||got - ref|| / ||ref|| <= 1e-13 (double-float keeps 48 significant bits; its
operator's error is of order 1e-14 of the site's terms).  The operator is the
reference's 64-bit one, lib/sse_su3dslash_64bit_scalar.c (4D) and
lib/sse_su3dslash_64bit_scalar_3d.c (3D)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

DF_TOL = 1e-13


@pytest.mark.parametrize("recon", [18, 12])
@pytest.mark.parametrize("nd,dims,layout_kind", [(4, (8, 4, 6, 4), "canonical"), (3, (4, 6, 4, 5), "canonical"),
                                                  (4, (4, 4, 2, 6), "scrambled"), (3, (4, 2, 4, 3), "scrambled")])
def test_double_float_matches_oracle(nd, dims, layout_kind, recon):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=nd, prec=64, recon=recon, spinor_format="double_float")
    V = op.volume
    if layout_kind == "canonical":
        lol = O.layout_table(O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D, dims)
    else:
        lol = O.scrambled_table(dims, 5)
        from sse_wilson_dslash_gb300.layouts import internal_coords
        x, y, z, t = internal_coords(dims, nd)
        lex = x + dims[0] * (y + dims[1] * (z + dims[2] * t))
        op.set_layout(lol[lex])
    u, psi = O.make_inputs(dims, 31, 32)
    gauge = op.pack_gauge(torch.from_numpy(np.ascontiguousarray(u)).cuda())
    pd = torch.from_numpy(np.ascontiguousarray(psi)).cuda()
    for isign in (1, -1):
        for cb in (0, 1):
            out = op.apply(gauge, op.pack_spinor(pd, cb), isign, cb)
            res = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
            err = O.site_rel_err(res.cpu().numpy(), ref, O.target_sites(nd, dims, lol, cb))
            assert err <= DF_TOL, (isign, cb, err)
    op.close()


@pytest.mark.parametrize("nd,dims", [(4, (8, 4, 6, 4)), (3, (4, 6, 4, 5)), (4, (2, 2, 2, 2)), (4, (6, 2, 2, 10))])
def test_double_float_variants_match_oracle(nd, dims):
    """Every variant: 0 the colour-split kernel (three warps a CTA, 32 sites;
    (6, 2, 2, 10) and (2, 2, 2, 2) leave the last CTA partly idle), 1-2 the
    one-thread-per-site kernel with register caps."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    lol = O.layout_table(O.LAYOUT_CB2 if nd == 4 else O.LAYOUT_CB3D, dims)
    u, psi = O.make_inputs(dims, 33, 34)
    for variant in range(3):
        op = DslashOperator(dims, nd=nd, prec=64, recon=18, spinor_format="double_float")
        op.set_tuning(0, variant)
        V = op.volume
        gauge = op.pack_gauge(torch.from_numpy(np.ascontiguousarray(u)).cuda())
        pd = torch.from_numpy(np.ascontiguousarray(psi)).cuda()
        for isign, cb in ((1, 1), (-1, 0)):
            out = op.apply(gauge, op.pack_spinor(pd, cb), isign, cb)
            res = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
            op.unpack_spinor(out, 1 - cb, res)
            ref = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
            err = O.site_rel_err(res.cpu().numpy(), ref, O.target_sites(nd, dims, lol, cb))
            assert err <= DF_TOL, (variant, isign, cb, err)
        op.close()


def test_double_float_pack_round_trip():
    """pack -> unpack keeps 48 significant bits of every double (relative
    error <= 2^-47) and FP32-representable values exactly."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (4, 4, 4, 6)
    op = DslashOperator(dims, nd=4, prec=64, spinor_format="double_float")
    rng = np.random.default_rng(5)
    V = op.volume
    psi = rng.standard_normal(V * 24) * np.exp(rng.uniform(-20, 20, V * 24))
    psi[::7] = psi[::7].astype(np.float32)
    pd = torch.from_numpy(psi).cuda()
    back = torch.zeros_like(pd)
    for parity in (0, 1):
        op.unpack_spinor(op.pack_spinor(pd, parity), parity, back)
    got = back.cpu().numpy()
    assert np.all(np.abs(got - psi) <= 2.0 ** -47 * np.abs(psi))
    assert np.array_equal(got[::7], psi[::7])
    op.close()


def test_double_float_agrees_with_fp64_on_24x24x24x48():
    """24^3x48 with random SU(3) links: the double-float and the FP64
    operators agree per site to 1e-13 on every target site (both checked
    against the oracle on the small lattices above)."""
    import torch
    from bench import su3_links
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (24, 24, 24, 48)
    V = 24 * 24 * 24 * 48
    gen = torch.Generator(device="cuda").manual_seed(41)
    u = su3_links(V * 4, gen, torch).reshape(-1)
    psi = torch.randn(V * 24, dtype=torch.float64, device="cuda", generator=gen)
    outs = {}
    for fmt in ("native", "double_float"):
        op = DslashOperator(dims, nd=4, prec=64, spinor_format=fmt)
        gauge = op.pack_gauge(u)
        src = op.pack_spinor(psi, 0)
        if fmt == "double_float":
            # the autotuner picks among the colour-split kernel and the
            # capped one-thread-per-site variants; any pick keeps the result
            threads, variant = op.autotune(gauge, src, op.new_spinor())
            assert 0 <= variant < op.num_variants
        out = op.apply(gauge, src, -1, 0)
        res = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
        op.unpack_spinor(out, 1, res)
        outs[fmt] = res.view(V, 24)
        op.close()
    a, b = outs["native"], outs["double_float"]
    nz = b.norm(dim=1) > 0
    assert int(nz.sum()) == V // 2
    rel = ((a - b).norm(dim=1)[nz] / a.norm(dim=1)[nz]).max().item()
    assert rel <= DF_TOL, rel


def test_double_float_rejects_what_it_does_not_cover():
    import torch
    from sse_wilson_dslash_gb300 import _lib
    from sse_wilson_dslash_gb300.device import DslashOperator
    for kw in (dict(prec=32), dict(prec=64, nrhs=2)):
        with pytest.raises(_lib.GbdsError):
            DslashOperator((4, 4, 4, 4), spinor_format="double_float", **kw)
    op = DslashOperator((4, 4, 4, 4), prec=64, spinor_format="double_float")
    f = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(_lib.GbdsError):
        op.pack_faces(op.new_gauge(), op.new_spinor(), 1, 0, f, f)
    with pytest.raises(_lib.GbdsError):
        op.force(op.new_gauge(), op.new_spinor(), op.new_spinor(), 1, 0,
                 torch.empty(op.volume * 72, dtype=torch.float64, device="cuda"))
    op.close()
