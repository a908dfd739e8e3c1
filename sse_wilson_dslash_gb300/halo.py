"""The lattice split along t across ranks: slab partition, face exchange and
the per-rank operator (gbds_op_pack_faces / gbds_op_dslash_halo in
include/gbdslash.h).

This is the GB300 form of the reference's parscalar build
(lib/sse_su3dslash_32bit_parscalar.c), where QMP moves the projected
half-spinor faces between nodes and the interior sites are computed while
they travel (:1203-1284).  Here each rank holds an equal slab of time slices
on its own GPU; the faces move with torch.distributed point-to-point calls
(NCCL on GPUs; any backend that moves the tensors works), and the interior
launch overlaps the exchange.  One rank (no process group) exchanges with
itself, which gives the periodic operator.
"""
from __future__ import annotations

TAG_TO_PREV, TAG_TO_NEXT = 11, 12


def slab(dims, world: int, rank: int):
    """(local dims, first global time slice) of ``rank``'s slab when the
    lattice ``dims`` is split along t into ``world`` equal slabs.  Each slab
    needs an even number of time slices, so that local and global parities
    agree."""
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world size or rank")
    if Lt % world:
        raise ValueError(f"Lt = {Lt} does not split into {world} equal slabs")
    lt = Lt // world
    if lt % 2:
        raise ValueError(f"a slab of {lt} time slices is odd; each rank needs an even number")
    return (Lx, Ly, Lz, lt), rank * lt


def exchange_faces(to_prev, to_next, from_prev, from_next, group=None, timeout=None):
    """Send ``to_prev`` to the previous rank (its ``from_next``) and
    ``to_next`` to the next rank (its ``from_prev``), periodic in the rank
    index; receive the neighbours' faces.  Blocks until the faces have
    arrived (for NCCL: until the current stream waits for them).  Without an
    initialised process group, or with one rank, the rank is its own
    neighbour.  A neighbour that left or never arrives makes the waits raise
    (RuntimeError) after ``timeout`` (a datetime.timedelta; default: the
    process group's timeout) instead of blocking for good."""
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
    if world == 1:
        from_next.copy_(to_prev)
        from_prev.copy_(to_next)
        return
    rank = dist.get_rank(group)
    prev, nxt = (rank - 1) % world, (rank + 1) % world
    if group is not None:
        prev, nxt = dist.get_global_rank(group, prev), dist.get_global_rank(group, nxt)
    # One group of four point-to-point operations (for NCCL one
    # ncclGroupStart/End, so no send waits on a receive queued behind it).
    # With two ranks prev == next: the two messages of the pair travel in the
    # order posted, which the receives follow, and the tags tell them apart
    # where the backend uses tags.
    ops = [dist.P2POp(dist.isend, to_prev, prev, group, TAG_TO_PREV),
           dist.P2POp(dist.isend, to_next, nxt, group, TAG_TO_NEXT),
           dist.P2POp(dist.irecv, from_next, nxt, group, TAG_TO_PREV),
           dist.P2POp(dist.irecv, from_prev, prev, group, TAG_TO_NEXT)]
    for r in dist.batch_isend_irecv(ops):
        if timeout is None:
            r.wait()
        else:
            r.wait(timeout)


class SplitDslash:
    """The Dslash of this rank's slab of a lattice split along t.

    Fields are the internal ones of ``self.op`` (a DslashOperator of the
    slab's local dims): pack with ``op.pack_gauge`` / ``op.pack_spinor`` from
    the slab's part of the packed arrays (local QDP++ cb2 order)."""

    def __init__(self, global_dims, prec: int = 32, recon: int = 18, group=None, device=None, timeout=None):
        """timeout: bound on the face exchange's waits (exchange_faces)."""
        import torch.distributed as dist
        from .device import DslashOperator
        self.group = group
        self.timeout = timeout
        self.world = dist.get_world_size(group) if dist.is_available() and dist.is_initialized() else 1
        self.rank = dist.get_rank(group) if self.world > 1 else 0
        self.global_dims = tuple(int(v) for v in global_dims)
        self.local_dims, self.t0 = slab(self.global_dims, self.world, self.rank)
        self.op = DslashOperator(self.local_dims, nd=4, prec=prec, recon=recon, device=device)
        self.to_prev, self.to_next = self.op.new_face(), self.op.new_face()
        self.from_prev, self.from_next = self.op.new_face(), self.op.new_face()
        self._comm = None

    def apply(self, gauge, psi, isign: int, cb: int, out=None, overlap: bool = True):
        """out (checkerboard 1-cb of the slab) = Dslash psi of the whole
        lattice restricted to this slab.  With ``overlap`` the interior time
        slices are computed on the current stream while the faces travel on a
        second one."""
        import torch
        op = self.op
        out = op.new_spinor() if out is None else out
        stream = torch.cuda.current_stream(op.device)
        op.pack_faces(gauge, psi, isign, cb, self.to_prev, self.to_next, stream=stream)
        if not overlap:
            exchange_faces(self.to_prev, self.to_next, self.from_prev, self.from_next, self.group, self.timeout)
            return op.apply_halo(gauge, psi, self.from_prev, self.from_next, isign, cb, out=out, part="all",
                                 stream=stream)
        if self._comm is None:
            self._comm = torch.cuda.Stream(op.device)
        self._comm.wait_stream(stream)
        with torch.cuda.stream(self._comm):
            exchange_faces(self.to_prev, self.to_next, self.from_prev, self.from_next, self.group, self.timeout)
        op.apply_halo(gauge, psi, None, None, isign, cb, out=out, part="interior", stream=stream)
        stream.wait_stream(self._comm)
        return op.apply_halo(gauge, psi, self.from_prev, self.from_next, isign, cb, out=out, part="boundary",
                             stream=stream)

    def close(self):
        self.op.close()
