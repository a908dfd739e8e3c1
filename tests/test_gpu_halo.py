"""The lattice split along t (GPU): gbds_op_pack_faces and
gbds_op_dslash_halo against the oracle.

One GPU plays every rank in turn: each slab has its own operator and
fields, its send faces are packed by the library's kernel, the "exchange"
is a device copy into the neighbours' receive buffers (what NCCL send/recv
does between GPUs), and the slab's output comes from one launch ('all') or
from the interior launch and the boundary launch.  The slabs' outputs,
put back into the whole lattice, are compared site by site with the oracle's
Dslash of the whole lattice (1e-6 FP32, 1e-13 FP64).  Reference:
lib/sse_su3dslash_32bit_parscalar.c:967-1284."""
import numpy as np
import pytest

import oracle as O
from golden_data import SITE_TOL
from halo_split import slab_sites

pytestmark = pytest.mark.gpu


def _run_split(dims, world, prec, recon, parts, u, psi, isign, cb, torch):
    from sse_wilson_dslash_gb300.device import DslashOperator
    from sse_wilson_dslash_gb300.halo import slab
    dt = torch.float32 if prec == 32 else torch.float64
    ranks = []
    for r in range(world):
        local, _ = slab(dims, world, r)
        op = DslashOperator(local, nd=4, prec=prec, recon=recon)
        sites = slab_sites(dims, world, r)
        gauge = op.pack_gauge(torch.from_numpy(np.ascontiguousarray(u[sites]).ravel()).to(dt).cuda())
        src = op.pack_spinor(torch.from_numpy(np.ascontiguousarray(psi[sites]).ravel()).to(dt).cuda(), cb)
        ranks.append(dict(op=op, sites=sites, gauge=gauge, src=src, to_prev=op.new_face(), to_next=op.new_face(),
                          from_prev=op.new_face(), from_next=op.new_face()))
    for R in ranks:
        R["op"].pack_faces(R["gauge"], R["src"], isign, cb, R["to_prev"], R["to_next"])
    for k, R in enumerate(ranks):  # the exchange: periodic in the rank index
        R["from_next"].copy_(ranks[(k + 1) % world]["to_prev"])
        R["from_prev"].copy_(ranks[(k - 1) % world]["to_next"])
    V = O.volume(dims)
    out = np.zeros((V, 24))
    for R in ranks:
        op = R["op"]
        res = op.new_spinor()
        if parts == "all":
            op.apply_halo(R["gauge"], R["src"], R["from_prev"], R["from_next"], isign, cb, out=res, part="all")
        else:
            op.apply_halo(R["gauge"], R["src"], None, None, isign, cb, out=res, part="interior")
            op.apply_halo(R["gauge"], R["src"], R["from_prev"], R["from_next"], isign, cb, out=res, part="boundary")
        packed = torch.zeros(op.volume * 24, dtype=dt, device="cuda")
        op.unpack_spinor(res, 1 - cb, packed)
        out[R["sites"]] = packed.double().cpu().numpy().reshape(-1, 24)
        op.close()
    return out


@pytest.mark.parametrize("parts", ["all", "split"])
@pytest.mark.parametrize("recon", [18, 12])
@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("world", [1, 2, 4])
def test_split_t_matches_oracle(world, prec, recon, parts):
    import torch
    dims = (8, 4, 6, 16)
    u, psi = O.make_inputs(dims, 61, 62)
    dt = np.float32 if prec == 32 else np.float64
    u, psi = u.astype(dt), psi.astype(dt)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    for isign, cb in ((1, 0), (-1, 1), (1, 1), (-1, 0)):
        got = _run_split(dims, world, prec, recon, parts, u, psi, isign, cb, torch)
        ref = O.dslash_plain(4, dims, lol, u, psi, isign, cb)
        err = O.site_rel_err(got, ref, O.target_sites(4, dims, lol, cb))
        assert err <= SITE_TOL[prec], (world, prec, recon, parts, isign, cb, err)


def test_two_time_slices_per_rank_has_no_interior():
    """Slabs of Lt = 2: every site is on a boundary slice; the interior
    launch does nothing and the boundary launch does all of them."""
    import torch
    dims = (4, 4, 4, 8)
    u, psi = O.make_inputs(dims, 63, 64)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    got = _run_split(dims, 4, 64, 18, "split", u, psi, -1, 0, torch)
    ref = O.dslash_plain(4, dims, lol, u, psi, -1, 0)
    assert O.site_rel_err(got, ref, O.target_sites(4, dims, lol, 0)) <= SITE_TOL[64]


@pytest.mark.parametrize("overlap", [True, False])
def test_split_dslash_single_rank_is_the_periodic_operator(overlap):
    """halo.SplitDslash without a process group: the rank is its own
    neighbour, and the result equals the periodic operator's (FP32, both
    launches of the overlapped form on the same stream order)."""
    import torch
    from sse_wilson_dslash_gb300.halo import SplitDslash
    dims = (8, 8, 4, 8)
    u, psi = O.make_inputs(dims, 65, 66)
    sd = SplitDslash(dims, prec=32, recon=18)
    op = sd.op
    gauge = op.pack_gauge(torch.from_numpy(u.astype(np.float32).ravel()).cuda())
    src = op.pack_spinor(torch.from_numpy(psi.astype(np.float32).ravel()).cuda(), 1)
    got = sd.apply(gauge, src, 1, 1, overlap=overlap)
    ref = op.apply(gauge, src, 1, 1)
    torch.cuda.synchronize()
    a = got.view(torch.float32)[: op.volume_cb * 24]
    b = ref.view(torch.float32)[: op.volume_cb * 24]
    assert (a - b).abs().max().item() <= 1e-6 * b.abs().max().item()
    sd.close()


def test_split_operator_rejects_unsupported_operators():
    from sse_wilson_dslash_gb300 import _lib
    from sse_wilson_dslash_gb300.device import DslashOperator
    import torch
    op = DslashOperator((4, 4, 4, 4), nd=4, prec=32, nrhs=8)
    f = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    with pytest.raises(_lib.GbdsError):
        op.pack_faces(op.new_gauge(), op.new_spinor(), 1, 0, f, f)
    op.close()
