"""Helpers for the split-t tests: the map between a global lattice's packed
arrays and each slab's (both in QDP++ cb2 order), and a numpy restatement of
one rank's halo Dslash (projected faces sent to the neighbours, the t hops
across the slab boundaries taken from the received ones)."""
import numpy as np

import oracle as O
from sse_wilson_dslash_gb300.halo import slab


def slab_sites(dims, world, rank):
    """Global packed index of each of the slab's sites, in the slab's packed
    (local cb2) order."""
    local, t0 = slab(dims, world, rank)
    Lx, Ly, Lz, lt = local
    glol = O.layout_table(O.LAYOUT_CB2, dims)
    llol = O.layout_table(O.LAYOUT_CB2, local)
    x, y, z, t = O.lex_coords(local)
    glex = x + Lx * (y + Ly * (z + Lz * (t + t0)))
    out = np.empty(O.volume(local), dtype=np.int64)
    out[llol[x + Lx * (y + Ly * (z + Lz * t))]] = glol[glex]
    return out


def faces_numpy(local, u, psi, isign, cb):
    """The two send buffers of a slab as complex arrays [Lz, Ly, Lx, 4, 3]
    (zero off the source checkerboard): to_prev = (1 - isign g_t) psi on the
    first time slice, to_next = U_t^+ (1 + isign g_t) psi on the last one."""
    lol = O.layout_table(O.LAYOUT_CB2, local)
    U, P = O.to_lex_fields(local, lol, u, psi)  # U[mu, t, z, y, x, i, j], P[t, z, y, x, s, c]
    g = O.gamma_matrices()[3]
    par = O.parity_of_lex(local, 4).reshape(P.shape[:4])
    src = (par == cb)[..., None, None]
    pm, pp = np.eye(4) - isign * g, np.eye(4) + isign * g
    to_prev = np.where(src[0], np.einsum("st,zyxtc->zyxsc", pm, P[0]), 0)
    w = np.einsum("st,zyxtc->zyxsc", pp, P[-1])
    to_next = np.where(src[-1], np.einsum("zyxji,zyxsj->zyxsi", np.conj(U[3, -1]), w), 0)
    return to_prev, to_next


def halo_dslash_numpy(local, u, psi, from_prev, from_next, isign, cb):
    """res of one slab (packed [V][4][3][2], target checkerboard only):
    x, y, z periodic within the slab, t hops across its first and last slices
    from the received faces."""
    lol = O.layout_table(O.LAYOUT_CB2, local)
    U, P = O.to_lex_fields(local, lol, u, psi)
    g = O.gamma_matrices()
    acc = np.zeros_like(P)
    axis = {0: 3, 1: 2, 2: 1}
    one = np.eye(4)
    for mu in range(3):
        pm, pp = one - isign * g[mu], one + isign * g[mu]
        acc += np.einsum("...ij,st,...tj->...si", U[mu], pm, np.roll(P, -1, axis=axis[mu]))
        w = np.einsum("...ji,st,...tj->...si", np.conj(U[mu]), pp, P)
        acc += np.roll(w, 1, axis=axis[mu])
    pm, pp = one - isign * g[3], one + isign * g[3]
    fwd = np.einsum("st,...tj->...sj", pm, np.concatenate([P[1:], np.zeros_like(P[:1])], axis=0))
    fwd[-1] = from_next
    acc += np.einsum("...ij,...sj->...si", U[3], fwd)
    bwd = np.einsum("...ji,st,...tj->...si", np.conj(U[3]), pp, P)
    bwd = np.concatenate([from_prev[None], bwd[:-1]], axis=0)
    acc += bwd
    V = O.volume(local)
    par = O.parity_of_lex(local, 4)
    sel = par == 1 - cb
    flat = acc.reshape(V, 4, 3)
    out = np.zeros((V, 4, 3, 2))
    out[lol[sel], ..., 0] = flat[sel].real
    out[lol[sel], ..., 1] = flat[sel].imag
    return out
