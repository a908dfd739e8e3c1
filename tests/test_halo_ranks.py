"""The lattice split along t across ranks, on the CPU: gloo processes (2 and
4 ranks) each hold one slab (sse_wilson_dslash_gb300.halo.slab), compute
their send faces, exchange them with halo.exchange_faces -- the function the
GPU ranks call with NCCL -- and apply the slab's operator with the received
faces (a numpy restatement of gbds_op_dslash_halo).  Every rank's output is
compared with the oracle's Dslash of the whole lattice on its slab.  The
same partition and face layout run on the GPU in test_gpu_halo.py."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, dims, results):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle as O
        from halo_split import faces_numpy, halo_dslash_numpy, slab_sites
        from sse_wilson_dslash_gb300.halo import exchange_faces, slab
        local, t0 = slab(dims, world, rank)
        u, psi = O.make_inputs(dims, 41, 42)  # every rank draws the whole lattice's inputs
        sites = slab_sites(dims, world, rank)
        lu, lpsi = u[sites], psi[sites]
        glol = O.layout_table(O.LAYOUT_CB2, dims)
        worst = 0.0
        for isign, cb in ((1, 0), (-1, 1), (1, 1), (-1, 0)):
            to_prev, to_next = faces_numpy(local, lu, lpsi, isign, cb)
            tp = torch.from_numpy(np.ascontiguousarray(to_prev).view(np.float64).copy())
            tn = torch.from_numpy(np.ascontiguousarray(to_next).view(np.float64).copy())
            fp, fn = torch.empty_like(tp), torch.empty_like(tn)
            exchange_faces(tp, tn, fp, fn)
            from_prev = fp.numpy().view(np.complex128).reshape(to_next.shape)
            from_next = fn.numpy().view(np.complex128).reshape(to_prev.shape)
            got = halo_dslash_numpy(local, lu, lpsi, from_prev, from_next, isign, cb)
            ref = O.dslash_plain(4, dims, glol, u, psi, isign, cb)[sites]
            lol = O.layout_table(O.LAYOUT_CB2, local)
            worst = max(worst, O.site_rel_err(got, ref, O.target_sites(4, local, lol, cb)))
        results[rank] = (t0, worst)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,dims", [(2, (4, 4, 2, 8)), (4, (4, 2, 4, 8))])
def test_split_ranks_match_the_oracle(world, dims):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    results = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, dims, results)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    lt = dims[3] // world
    for r in range(world):
        t0, err = results[r]
        assert t0 == r * lt
        assert err < 1e-13, (r, err)


def _rank_leaves(rank, world, port, results):
    """Rank 1 leaves between steps (it never posts its half of the
    exchange); rank 0's exchange must raise within the bounded wait."""
    import datetime
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    try:
        from sse_wilson_dslash_gb300.halo import exchange_faces
        if rank == 1:
            results[rank] = "left"
            return
        faces = [torch.zeros(96, dtype=torch.float64) for _ in range(4)]
        try:
            exchange_faces(*faces, timeout=datetime.timedelta(seconds=3))
            results[rank] = "completed"
        except RuntimeError:
            results[rank] = "raised"
    finally:
        dist.destroy_process_group()


def test_a_rank_that_leaves_makes_the_exchange_raise():
    """The failure is made on the host, as the split-t path's failure tests
    are: one gloo rank leaves before the face exchange; the other's
    exchange_faces raises RuntimeError within its bounded wait and the
    process ends normally (no hang, no abort)."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    results = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_leaves, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert results[1] == "left"
    assert results[0] == "raised"


def test_slab_partition_rules():
    from sse_wilson_dslash_gb300.halo import slab
    assert slab((8, 8, 8, 16), 4, 3) == ((8, 8, 8, 4), 12)
    assert slab((4, 4, 4, 4), 1, 0) == ((4, 4, 4, 4), 0)
    with pytest.raises(ValueError, match="equal slabs"):
        slab((4, 4, 4, 12), 5, 0)
    with pytest.raises(ValueError, match="odd"):
        slab((4, 4, 4, 12), 4, 0)  # 3 time slices a rank
    with pytest.raises(ValueError):
        slab((4, 4, 4, 8), 2, 2)
