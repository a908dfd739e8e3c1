"""Test-only torch.autograd.Function around the library's Dslash and its
hand-written adjoint (gbds_op_dslash with -isign for dL/dpsi, gbds_op_force
mode 0 for dL/dU).  Not part of the product."""
import torch


class DslashFn(torch.autograd.Function):
    """res = Dslash(isign) psi on the sites of checkerboard 1-cb (zero
    elsewhere); u, psi, res are packed float64/float32 CUDA tensors
    ([V][4][3][3][2], [V][4][3][2], QDP++ cb2 order)."""

    @staticmethod
    def forward(ctx, u, psi, op, isign, cb):
        gauge = op.pack_gauge(u)
        src = op.pack_spinor(psi, cb)
        out = op.apply(gauge, src, isign, cb)
        res = torch.zeros_like(psi)
        op.unpack_spinor(out, 1 - cb, res)
        ctx.save_for_backward(u, psi)
        ctx.op, ctx.isign, ctx.cb, ctx.gauge, ctx.src = op, isign, cb, gauge, src
        return res

    @staticmethod
    def backward(ctx, grad_res):
        op, isign, cb = ctx.op, ctx.isign, ctx.cb
        u, psi = ctx.saved_tensors
        chi = op.pack_spinor(grad_res.contiguous(), 1 - cb)
        grad_psi = torch.zeros_like(psi)
        op.unpack_spinor(op.apply(ctx.gauge, chi, -isign, 1 - cb), cb, grad_psi)
        grad_u = torch.zeros_like(u)
        op.force(ctx.gauge, ctx.src, chi, isign, cb, grad_u, mode=0)
        return grad_u, grad_psi, None, None, None
