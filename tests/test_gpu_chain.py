"""Back-to-back dependent applications on one stream, and the same pair
replayed from a CUDA graph, against the oracle.

The second application reads the first one's output.  The Dslash kernels
are launched with programmatic dependent launch: a grid may be dispatched
while the previous one is still running and must wait for it before its
first global read.  These tests check that ordering with lattices of more
blocks than the GPU holds at once (single rhs) and with a multi-RHS kernel
whose grid fits at once, so that the dependent grid is resident while the
first one runs."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

# (dims, prec, nrhs, spinor format, kernel variant or None, per-site tolerance
# after two applications)
CASES = [
    ((16, 16, 16, 64), 32, 1, "native", None, 2e-6),
    ((16, 8, 8, 16), 64, 1, "native", None, 2e-13),
    ((8, 8, 8, 16), 32, 16, "f32_pairs", 2, 2e-6),
    ((8, 8, 8, 16), 32, 16, "native", 1, 2e-6),
]


def _setup(dims, prec, nrhs, fmt, variant, seed):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    V = O.volume(dims)
    rng = np.random.default_rng(seed)
    u = O.random_gauge(rng, V)
    psis = [O.gaussian_spinor(rng, V) for _ in range(nrhs)]
    real = np.float32 if prec == 32 else np.float64
    op = DslashOperator(dims, nd=4, prec=prec, recon=18, nrhs=nrhs, spinor_format=fmt)
    if variant is not None:
        op.set_tuning(0, variant)
    gauge = op.pack_gauge(torch.from_numpy(u.astype(real).ravel()).cuda())
    src = op.pack_spinor(torch.from_numpy(np.stack(psis).astype(real).ravel()).cuda(), 0)
    return op, gauge, src, u.astype(real).astype(np.float64), [p.astype(real).astype(np.float64) for p in psis]


def _check(op, out2, dims, nrhs, prec, u, psis, isign, tol):
    import torch
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    res = torch.zeros(nrhs * V * 24, dtype=torch.float32 if prec == 32 else torch.float64, device="cuda")
    op.unpack_spinor(out2, 0, res)
    got = res.cpu().numpy().reshape(nrhs, V, 24)
    ts = O.target_sites(4, dims, lol, 1)
    for r in range(nrhs):
        mid = O.dslash_plain(4, dims, lol, u, psis[r], isign, 0)
        ref = O.dslash_plain(4, dims, lol, u, mid, isign, 1)
        err = O.site_rel_err(got[r], ref, ts)
        assert err <= tol, (r, err)


@pytest.mark.parametrize("dims,prec,nrhs,fmt,variant,tol", CASES)
def test_dependent_pair_matches_oracle(dims, prec, nrhs, fmt, variant, tol):
    op, gauge, src, u, psis = _setup(dims, prec, nrhs, fmt, variant, 17)
    for isign in (1, -1):
        mid = op.apply(gauge, src, isign, 0)
        out2 = op.apply(gauge, mid, isign, 1)
        _check(op, out2, dims, nrhs, prec, u, psis, isign, tol)
    op.close()


@pytest.mark.parametrize("dims,prec,nrhs,fmt,variant,tol", [CASES[0], CASES[2]])
def test_dependent_pair_replayed_from_a_graph(dims, prec, nrhs, fmt, variant, tol):
    import torch
    op, gauge, src, u, psis = _setup(dims, prec, nrhs, fmt, variant, 23)
    mid, out2 = op.new_spinor(), op.new_spinor()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # warm-up outside the capture
        op.apply(gauge, src, 1, 0, out=mid, stream=s)
        op.apply(gauge, mid, 1, 1, out=out2, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        cs = torch.cuda.current_stream()
        op.apply(gauge, src, 1, 0, out=mid, stream=cs)
        op.apply(gauge, mid, 1, 1, out=out2, stream=cs)
    mid.zero_()
    out2.zero_()
    torch.cuda.synchronize()
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    _check(op, out2, dims, nrhs, prec, u, psis, 1, tol)
    del g
    op.close()
