"""The largest lattice in the tests (GPU): 64^3x128, 33.5 M sites (gauge field
9.7 GB in FP32), built as the 4 x 4 x 4 x 4 tiling of a 16^3x32 lattice.
With periodic boundaries its Dslash is the same tiling of the small
lattice's Dslash, so every one of its 16.8 M output sites is checked against
the small operator's output at the corresponding site (the small lattice is
itself checked against the oracle in the other tests, and one of its
applications again here).  This exercises the index arithmetic of the packing
and Dslash kernels at sizes where element offsets pass 2^31."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SMALL = (16, 16, 16, 32)
TILES = 4
BIG = tuple(TILES * v for v in SMALL)


def _cb2_index(dims, torch):
    """cb2 linear index of every lexicographic site (lex = x + Lx (y + Ly (z + Lz t)))."""
    Lx, Ly, Lz, Lt = dims
    lex = torch.arange(Lx * Ly * Lz * Lt, device="cuda", dtype=torch.int64)
    x, y, z, t = lex % Lx, (lex // Lx) % Ly, (lex // (Lx * Ly)) % Lz, lex // (Lx * Ly * Lz)
    p = (x + y + z + t) & 1
    return p * (lex.numel() // 2) + ((t * Lz + z) * Ly + y) * (Lx // 2) + x // 2


def _tile_lex(a, torch):
    """[Lt, Lz, Ly, Lx, k] of SMALL -> the same tiled to BIG."""
    return a.repeat(TILES, TILES, TILES, TILES, 1)


def _to_packed(lex, dims, torch):
    """lexicographic [V, k] -> packed cb2 order [V, k]."""
    out = torch.empty_like(lex)
    out[_cb2_index(dims, torch)] = lex
    return out


def _from_packed(packed, dims, torch):
    return packed[_cb2_index(dims, torch)]


@pytest.mark.slow
@pytest.mark.parametrize("isign,cb", [(1, 0), (-1, 1)])
def test_64x64x64x128_is_the_tiling_of_16x16x16x32(isign, cb):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    Ls = SMALL[::-1]  # (Lt, Lz, Ly, Lx)
    gen = torch.Generator(device="cuda").manual_seed(77)
    u_small = torch.randn(*Ls, 72, device="cuda", generator=gen)     # any links: recon 18
    psi_small = torch.randn(*Ls, 24, device="cuda", generator=gen)

    def run(dims, u_lex, psi_lex):
        op = DslashOperator(dims, nd=4, prec=32, recon=18)
        op.set_tuning(128, 1)  # the same kernel for both lattices
        V = op.volume
        gauge = op.pack_gauge(_to_packed(u_lex.reshape(V, 72), dims, torch).reshape(-1))
        src = op.pack_spinor(_to_packed(psi_lex.reshape(V, 24), dims, torch).reshape(-1), cb)
        out = op.apply(gauge, src, isign, cb)
        del gauge, src
        packed = torch.zeros(V * 24, device="cuda")
        op.unpack_spinor(out, 1 - cb, packed)
        op.close()
        return _from_packed(packed.view(V, 24), dims, torch)  # lexicographic [V, 24]

    small = run(SMALL, u_small, psi_small)
    # the small lattice against the oracle
    V = O.volume(SMALL)
    lol = O.layout_table(O.LAYOUT_CB2, SMALL)
    u_np = _to_packed(u_small.reshape(V, 72), SMALL, torch).cpu().numpy()
    p_np = _to_packed(psi_small.reshape(V, 24), SMALL, torch).cpu().numpy()
    ref = O.dslash_plain(4, SMALL, lol, u_np, p_np, isign, cb)
    got = _to_packed(small, SMALL, torch).cpu().numpy()
    assert O.site_rel_err(got, ref, O.target_sites(4, SMALL, lol, cb)) <= 1e-6
    # the big lattice against the tiled small one, every site
    big = run(BIG, _tile_lex(u_small, torch), _tile_lex(psi_small, torch))
    want = _tile_lex(small.view(*Ls, 24), torch).reshape(-1, 24)
    assert big.shape == want.shape
    assert torch.equal(big, want)
