"""Uneven batches in one persistent launch (GPU): every lattice of the batch
gives the same result as its own operator, directly and through a captured
CUDA graph; runtime right-hand-side counts against the oracle."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _item(dims, nrhs, isign, cb, recon, fmt, seed, torch):
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=4, prec=32, recon=recon, nrhs=nrhs, spinor_format=fmt)
    g = torch.Generator(device="cuda").manual_seed(seed)
    V = op.volume
    u = torch.from_numpy(O.random_gauge(np.random.default_rng(seed), V).astype(np.float32).ravel()).cuda()
    psi = torch.randn(nrhs * V * 24, dtype=torch.float32, device="cuda", generator=g)
    gauge = op.pack_gauge(u)
    src = op.pack_spinor(psi, cb)
    ref = op.apply(gauge, src, isign, cb)
    return dict(op=op, gauge=gauge, psi=src, res=op.new_spinor(), isign=isign, cb=cb, ref=ref)


# The batch kernel and the per-operator kernel do the same arithmetic in the
# same order, but the compiler may contract multiply-adds differently in the
# two kernels: FP32 results agree to rounding, and a rounding difference can
# move a 16-bit stored value by one unit.
TOL = {"native": 1e-5, "f32_pairs": 1e-5, "bf16": 1e-2, "f16": 2e-3}


def _same(op, a, b, fmt):
    import torch
    fa = torch.zeros(op.nrhs * op.volume * 24, dtype=torch.float32, device="cuda")
    fb = torch.zeros_like(fa)
    op.unpack_spinor(a, 0, fa)
    op.unpack_spinor(a, 1, fa)
    op.unpack_spinor(b, 0, fb)
    op.unpack_spinor(b, 1, fb)
    return float((fa - fb).abs().max()) <= TOL[fmt] * float(fb.abs().max())


@pytest.mark.parametrize("recon,fmt", [(18, "native"), (12, "native"), (18, "bf16"), (12, "f16"), (18, "f32_pairs")])
def test_batch_matches_single_operators(recon, fmt):
    import torch
    from sse_wilson_dslash_gb300.device import DslashBatch
    specs = [((4, 4, 4, 4), 1, 1, 0), ((6, 4, 4, 2), 3, -1, 1), ((8, 4, 2, 4), 8, 1, 1), ((4, 2, 6, 4), 5, -1, 0),
             ((2, 2, 2, 2), 2, 1, 0)]
    items = [_item(d, n, s, c, recon, fmt, 10 + k, torch) for k, (d, n, s, c) in enumerate(specs)]
    b = DslashBatch(items, recon=recon, spinor_format=fmt)
    for it in items:
        it["res"].zero_()
    b.launch()
    torch.cuda.synchronize()
    for it in items:
        assert _same(it["op"], it["res"], it["ref"], fmt)
    sch = b.autotune()
    assert sch["tile_threads"] in (64, 128, 256) and sch["tiles"] > 0
    for it in items:
        it["res"].zero_()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.capture_graph(s)
        for _ in range(2):
            b.launch(s)
    s.synchronize()
    for it in items:
        assert _same(it["op"], it["res"], it["ref"], fmt)
    b.close()


@pytest.mark.parametrize("nrhs", [3, 5, 7])
def test_runtime_nrhs_matches_oracle(nrhs):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (4, 4, 2, 6)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    rng = np.random.default_rng(nrhs)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    op = DslashOperator(dims, prec=32, nrhs=nrhs)
    gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
    src = op.pack_spinor(torch.from_numpy(np.stack(psis).astype(np.float32).ravel()).cuda(), 1)
    out = op.apply(gauge, src, -1, 1)
    res = torch.zeros(nrhs * V * 24, dtype=torch.float32, device="cuda")
    op.unpack_spinor(out, 0, res)
    got = res.cpu().numpy().reshape(nrhs, V, 24)
    ts = O.target_sites(4, dims, lol, 1)
    for r in range(nrhs):
        ref = O.dslash_plain(4, dims, lol, u.astype(np.float32), psis[r].astype(np.float32), -1, 1)
        assert O.site_rel_err(got[r], ref, ts) <= 1e-6
