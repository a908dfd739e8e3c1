"""The portable SSE shim (oracle/sse_shim/xmmintrin.h) that lets the
reference scalar library be compiled from its own sources on hosts without
x86 SSE: where both builds exist (x86_64 with the reference sources), the
shim build gives the native SSE build's results bit for bit, for the 4D and
3D operators in FP32 and FP64, every isign and cb (CPU only).

Each (library, operator) runs in a fresh process: the reference keeps one
lattice per library in global state, and its FP64 3D free also frees the 4D
tables (lib/sse_su3dslash_64bit_scalar_3d.c:128)."""
import multiprocessing as mp

import numpy as np
import pytest

import oracle as O

CASES = [(4, (8, 8, 8, 8), O.LAYOUT_CB2), (4, (4, 2, 6, 8), O.LAYOUT_CB2), (3, (4, 6, 4, 5), O.LAYOUT_CB3D)]


def _run(prec, shim, nd, dims, kind, q):
    import oracle as O2
    R = O2.Reference(prec, shim=shim)
    R.init(nd, dims, kind)
    u, psi = O2.make_inputs(dims, 31, 32)
    dt = np.float32 if prec == 32 else np.float64
    u, psi = u.astype(dt), psi.astype(dt)
    outs = []
    for isign in (1, -1):
        for cb in (0, 1):
            res = np.zeros_like(psi)
            R.apply(nd, u, psi, res, isign, cb)
            outs.append(res)
    q.put(np.stack(outs))


def _outputs(prec, shim, nd, dims, kind):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_run, args=(prec, shim, nd, dims, kind, q))
    p.start()
    out = q.get(timeout=120)
    p.join(timeout=60)
    assert p.exitcode == 0
    return out


@pytest.mark.parametrize("nd,dims,kind", CASES)
@pytest.mark.parametrize("prec", [32, 64])
def test_shim_build_equals_native_sse_build(prec, nd, dims, kind):
    if not (O.reference_available(prec) and O.reference_available(prec, shim=True)):
        pytest.skip("needs the native and the shim build of the reference (x86_64 with its sources)")
    native = _outputs(prec, False, nd, dims, kind)
    shim = _outputs(prec, True, nd, dims, kind)
    assert np.any(native != 0)
    np.testing.assert_array_equal(native, shim)
