"""Uneven batches in one persistent launch (GPU).  Every lattice and every
right-hand side of a batch is checked against the oracle (orc_dslash_plain,
FP64) on the same inputs, directly, after the autotuner and from a captured
CUDA graph; the configured batch {16^4 x 8 rhs, 20^3x40 x 4, 24^3x48 x 2,
32^3x64 x 1} runs through the graph-replayed launch; two batches chained on
one stream (the second reads the first one's output) stay ordered.  The
operator is the reference's, lib/sse_su3dslash_32bit_scalar.c:185-293, per
lattice and right-hand side."""
import numpy as np
import pytest

import oracle as O
from formats import TOL, site_err, stored

pytestmark = pytest.mark.gpu


def _host_inputs(dims, nrhs, seed, torch):
    """Packed FP32 links [V][4][3][3][2] and spinors [nrhs][V][4][3][2]:
    random SU(3) links and N(0,1) spinors generated on the device."""
    from bench import su3_links
    V = O.volume(dims)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    u = su3_links(V * 4, gen, torch).float().reshape(V, 4, 3, 3, 2)
    psi = torch.randn(nrhs, V, 4, 3, 2, dtype=torch.float32, device="cuda", generator=gen)
    return u, psi


def _item(dims, nrhs, isign, cb, recon, fmt, seed, torch):
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=4, prec=32, recon=recon, nrhs=nrhs, spinor_format=fmt)
    u, psi = _host_inputs(dims, nrhs, seed, torch)
    gauge = op.pack_gauge(u.reshape(-1))
    src = op.pack_spinor(psi.reshape(-1), cb)
    return dict(op=op, gauge=gauge, psi=src, res=op.new_spinor(), isign=isign, cb=cb,
                u=u.cpu().numpy(), psi_host=psi.cpu().numpy(), fmt=fmt)


def _unpack(it, buf, parity, torch):
    op = it["op"]
    out = torch.zeros(op.nrhs * op.volume * 24, dtype=torch.float32, device="cuda")
    op.unpack_spinor(buf, parity, out)
    return out.view(op.nrhs, op.volume, 24).cpu().numpy()


def _oracle_refs(it, rhs):
    """Oracle outputs (FP64) of the item's rhs in ``rhs``: [len(rhs)][V][24]."""
    op = it["op"]
    lol = O.layout_table(O.LAYOUT_CB2, op.dims)
    src = stored(it["psi_host"][list(rhs)], it["fmt"])
    return np.stack([O.dslash_plain(4, op.dims, lol, it["u"], src[k], it["isign"], it["cb"]).reshape(op.volume, 24)
                     for k in range(len(rhs))])


def _check_items(items, torch, rhs_of=lambda it: range(it["op"].nrhs), refs=None):
    errs = []
    for k, it in enumerate(items):
        op = it["op"]
        rhs = list(rhs_of(it))
        got = _unpack(it, it["res"], 1 - it["cb"], torch)[rhs]
        ref = refs[k] if refs is not None else _oracle_refs(it, rhs)
        lol = O.layout_table(O.LAYOUT_CB2, op.dims)
        err = site_err(got, ref, O.target_sites(4, op.dims, lol, it["cb"]))
        errs.append(err)
        assert err <= TOL[it["fmt"]], (op.dims, op.nrhs, it["fmt"], err)
    return errs


@pytest.mark.parametrize("recon,fmt", [(18, "native"), (12, "native"), (18, "bf16"), (12, "f16"), (18, "f32_pairs")])
def test_batch_matches_oracle(recon, fmt):
    """Five lattices of different shapes, right-hand-side counts, isign and cb
    (runtime counts 3 and 5 among them): the plain launch, the autotuned
    schedule and the graph replay all agree with the oracle on every site and
    right-hand side."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashBatch
    specs = [((4, 4, 4, 4), 1, 1, 0), ((6, 4, 4, 2), 3, -1, 1), ((8, 4, 2, 4), 8, 1, 1), ((4, 2, 6, 4), 5, -1, 0),
             ((2, 2, 2, 2), 2, 1, 0)]
    items = [_item(d, n, s, c, recon, fmt, 10 + k, torch) for k, (d, n, s, c) in enumerate(specs)]
    refs = [_oracle_refs(it, range(it["op"].nrhs)) for it in items]
    b = DslashBatch(items, recon=recon, spinor_format=fmt)
    for it in items:
        it["res"].zero_()
    b.launch()
    torch.cuda.synchronize()
    _check_items(items, torch, refs=refs)
    sch = b.autotune()
    assert sch["tile_threads"] in (64, 128, 256) and sch["tiles"] > 0
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.capture_graph(s)
        for it in items:
            it["res"].zero_()
        for _ in range(2):
            b.launch(s)
    s.synchronize()
    _check_items(items, torch, refs=refs)
    b.close()


@pytest.mark.slow
def test_configured_uneven_batch_graph_against_oracle():
    """The configured batch -- 16^4 with 8 rhs, 20^3x40 with 4, 24^3x48 with
    2, 32^3x64 with 1, each with its own random SU(3) field -- autotuned and
    replayed from a CUDA graph; every rhs of the three smaller lattices and
    the one rhs of 32^3x64 against the oracle."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashBatch
    specs = [((16, 16, 16, 16), 8, 1, 0), ((20, 20, 20, 40), 4, -1, 1), ((24, 24, 24, 48), 2, 1, 1),
             ((32, 32, 32, 64), 1, -1, 0)]
    items = [_item(d, n, s, c, 18, "native", 80 + k, torch) for k, (d, n, s, c) in enumerate(specs)]
    b = DslashBatch(items)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.autotune(s)
        b.capture_graph(s)
        for it in items:
            it["res"].zero_()
        b.launch(s)
    s.synchronize()
    errs = _check_items(items, torch)
    assert max(errs) <= 1e-6
    b.close()


def test_two_batches_chained_on_one_stream():
    """A second batch reads the first one's output as its source: launched
    back to back on one stream, directly and from captured graphs, it sees the
    finished output (programmatic dependent launch waits for the previous
    grid).  Checked against the oracle applied to the first batch's result."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashBatch
    specs = [((8, 8, 4, 8), 4, 1, 0), ((6, 4, 4, 6), 2, -1, 1)]
    first = [_item(d, n, s, c, 18, "native", 90 + k, torch) for k, (d, n, s, c) in enumerate(specs)]
    second = []
    for it in first:
        # source: the first batch's output (checkerboard 1 - cb); the second
        # batch writes checkerboard cb
        second.append(dict(op=it["op"], gauge=it["gauge"], psi=it["res"], res=it["op"].new_spinor(),
                           isign=-it["isign"], cb=1 - it["cb"], u=it["u"], fmt="native"))
    b1 = DslashBatch(first)
    b2 = DslashBatch(second)
    s = torch.cuda.Stream()

    def run_and_check():
        s.synchronize()
        for it1, it2 in zip(first, second):
            op = it1["op"]
            lol = O.layout_table(O.LAYOUT_CB2, op.dims)
            mid = _unpack(it1, it1["res"], 1 - it1["cb"], torch)
            got = _unpack(it2, it2["res"], 1 - it2["cb"], torch)
            ref = np.stack([O.dslash_plain(4, op.dims, lol, it1["u"], mid[r].reshape(op.volume, 4, 3, 2),
                                           it2["isign"], it2["cb"]).reshape(op.volume, 24) for r in range(op.nrhs)])
            assert site_err(got, ref, O.target_sites(4, op.dims, lol, it2["cb"])) <= 1e-6
            first_ref = _oracle_refs(it1, range(op.nrhs))
            assert site_err(mid, first_ref, O.target_sites(4, op.dims, lol, it1["cb"])) <= 1e-6

    with torch.cuda.stream(s):
        for it in first + second:
            it["res"].zero_()
        b1.launch(s)
        b2.launch(s)
    run_and_check()
    with torch.cuda.stream(s):
        b1.capture_graph(s)
        b2.capture_graph(s)
        for _ in range(2):
            for it in first + second:
                it["res"].zero_()
            b1.launch(s)
            b2.launch(s)
    run_and_check()
    b1.close()
    b2.close()


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
