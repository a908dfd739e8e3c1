"""The oracle pinned against the reference's outputs (golden vectors), and
its restatements against each other.  CPU only."""
import numpy as np
import pytest

import oracle as O
from golden_data import check_against_golden, checksum_weights, layout, load

MAN, ARR = load()
CASES = sorted(MAN["cases"])


@pytest.mark.parametrize("name", CASES)
def test_generators_reproduce_golden_inputs(name):
    c = MAN["cases"][name]
    u, psi = O.make_inputs(c["dims"], MAN["seeds"]["gauge"], MAN["seeds"]["spinor"], c["gauge"])
    for arr, key in ((u, "u"), (psi, "psi")):
        s = float(np.dot(checksum_weights(arr.size), arr.ravel()))
        assert abs(s - c["input_checksums"][key]) <= 1e-12 * np.abs(arr).sum()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", [32, 64])
def test_plain_oracle_matches_reference(name, prec):
    c = MAN["cases"][name]
    dims, nd = c["dims"], c["nd"]
    _, lol = layout(c, dims)
    u, psi = O.make_inputs(dims, MAN["seeds"]["gauge"], MAN["seeds"]["spinor"], c["gauge"])
    dt = np.float32 if prec == 32 else np.float64
    u, psi = u.astype(dt), psi.astype(dt)
    for isign in (1, -1):
        for cb in (0, 1):
            res = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
            check_against_golden(MAN, ARR, name, prec, isign, cb, res)


@pytest.mark.parametrize("name", ["cb2_4x4x4x4", "cb3d_4x2x4x5", "perm_4x4x2x4", "cb2layout_3d_4x4x2x4"])
def test_numpy_and_port_restatements_agree(name):
    c = MAN["cases"][name]
    dims, nd = c["dims"], c["nd"]
    _, lol = layout(c, dims)
    u, psi = O.make_inputs(dims, MAN["seeds"]["gauge"], MAN["seeds"]["spinor"], c["gauge"])
    tabs = O.PortTables(nd, dims, lol)
    V = O.volume(dims)
    for isign in (1, -1):
        for cb in (0, 1):
            a = O.dslash_plain(nd, dims, lol, u, psi, isign, cb)
            b = O.dslash_numpy(nd, dims, lol, u, psi, isign, cb)
            p = np.zeros((V, 4, 3, 2))
            tabs.apply(u, psi, p, isign, cb, nthreads=2)
            ts = O.target_sites(nd, dims, lol, cb)
            assert O.site_rel_err(b, a, ts) < 1e-14
            assert O.site_rel_err(p, a, ts) < 1e-14
            p32 = np.zeros((V, 4, 3, 2), np.float32)
            tabs.apply(u.astype(np.float32), psi.astype(np.float32), p32, isign, cb, nthreads=2)
            assert O.site_rel_err(p32, a, ts) < 1e-6


def test_untouched_parity_and_bad_isign():
    dims = (4, 4, 4, 4)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, psi = O.make_inputs(dims)
    V = O.volume(dims)
    sentinel = np.full((V, 4, 3, 2), 7.0)
    out = O.dslash_plain(4, dims, lol, u, psi, 1, 0, res=sentinel)
    other = O.target_sites(4, dims, lol, 1)  # parity-0 sites (cb=1 writes them)
    assert np.all(out.reshape(V, 24)[other] == 7.0)
    assert np.all(O.dslash_plain(4, dims, lol, u, psi, 0, 0, res=sentinel) == 7.0)
    assert np.all(O.dslash_plain(4, dims, lol, u, psi, 2, 1, res=sentinel) == 7.0)


def test_gamma_algebra():
    g = O.gamma_matrices()
    one = np.eye(4)
    for m in range(4):
        assert np.allclose(g[m] @ g[m], one)
        assert np.allclose(g[m], g[m].conj().T)
        for n in range(m + 1, 4):
            assert np.allclose(g[m] @ g[n] + g[n] @ g[m], 0)


def test_generated_links_are_su3():
    rng = np.random.default_rng(0)
    for U in (O.random_su3(rng, 64), O.near_unit_su3(rng, 64)):
        eye = np.einsum("nij,nkj->nik", U, U.conj())
        assert np.allclose(eye, np.eye(3), atol=1e-13)
        assert np.allclose(np.linalg.det(U), 1, atol=1e-13)


def test_layout_callbacks_are_inverse():
    for kind, dims in ((O.LAYOUT_CB2, (4, 2, 6, 4)), (O.LAYOUT_CB3D, (4, 2, 6, 3)), (O.LAYOUT_LEX, (2, 2, 4, 2))):
        lol = O.layout_table(kind, dims)
        assert sorted(lol.tolist()) == list(range(O.volume(dims)))
