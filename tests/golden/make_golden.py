"""Generate the golden vectors that pin the oracle to the reference library.

Run from the repository root, on an x86_64 host that has the reference
sources (the reference library is compiled from them by ``oracle/Makefile``
into ``oracle/_ref``)::

    python tests/golden/make_golden.py

For every case below the script builds seeded inputs with the oracle's
generators, runs the reference's own ``sse_su3dslash_wilson`` /
``sse_su3dslash_wilson_3d`` (FP32 and FP64 library builds) for all four
(isign, cb) combinations through the reference's init/apply/free API, and
stores, per combination:

* ``sum`` and ``sumsq``: a weighted checksum of the whole output array
  (weights from :func:`checksum_weights`, exact in binary) and its squared
  norm -- these pin every site;
* the outputs at 32 sampled target sites (every target site for the cases
  marked ``full``), for per-site comparisons;
* a checksum of the inputs, so that a drift of the generators is caught.

The reference keeps one global lattice per library and its FP64 3D ``free``
also frees the 4D site table (lib/sse_su3dslash_64bit_scalar_3d.c:128), so
every (case, precision) runs in a fresh process.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

OUT_DIR = os.path.dirname(os.path.abspath(__file__))

# name, nd, dims, layout, gauge kind, store full outputs
CASES = [
    ("cb2_8x8x8x8", 4, (8, 8, 8, 8), "cb2", "haar", False),
    ("cb2_4x4x4x4", 4, (4, 4, 4, 4), "cb2", "haar", True),
    ("cb2_2x4x6x8", 4, (2, 4, 6, 8), "cb2", "haar", False),
    ("cb2_4x4x4x4_nearunit", 4, (4, 4, 4, 4), "cb2", "near_unit", False),
    ("lex_4x2x2x6", 4, (4, 2, 2, 6), "lex", "haar", False),
    ("perm_4x4x2x4", 4, (4, 4, 2, 4), "perm", "haar", False),
    ("cb3d_4x4x4x6", 3, (4, 4, 4, 6), "cb3d", "haar", True),
    ("cb3d_4x2x4x5", 3, (4, 2, 4, 5), "cb3d", "haar", False),
    ("cb3d_8x8x8x8", 3, (8, 8, 8, 8), "cb3d", "haar", False),
    ("cb2layout_3d_4x4x2x4", 3, (4, 4, 2, 4), "cb2", "haar", False),
]
SEED_GAUGE, SEED_SPINOR, SEED_PERM = 1234, 5678, 7
N_SAMPLE = 32


def checksum_weights(n: int) -> np.ndarray:
    """Weights in [-0.5, 0.5) from an integer hash; exact in binary on every
    platform (a multiple of 2**-32)."""
    k = np.arange(n, dtype=np.uint64)
    h = (k * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(2 ** 32)
    return h.astype(np.float64) / 2.0 ** 32 - 0.5


def layout_for(name: str, dims):
    import oracle as O
    if name == "cb2":
        return O.LAYOUT_CB2, O.layout_table(O.LAYOUT_CB2, dims)
    if name == "cb3d":
        return O.LAYOUT_CB3D, O.layout_table(O.LAYOUT_CB3D, dims)
    if name == "lex":
        return O.LAYOUT_LEX, O.layout_table(O.LAYOUT_LEX, dims)
    if name == "perm":
        return O.LAYOUT_PERM, O.scrambled_table(dims, SEED_PERM)
    raise ValueError(name)


def sample_sites(nd, dims, lol, cb, full):
    import oracle as O
    ts = np.sort(O.target_sites(nd, dims, lol, cb))
    if full or len(ts) <= N_SAMPLE:
        return ts
    rng = np.random.default_rng(4321 + cb)
    return np.sort(rng.choice(ts, N_SAMPLE, replace=False))


def run_case(args):
    name, nd, dims, layout, gkind, full, prec = args
    import oracle as O
    kind, lol = layout_for(layout, dims)
    V = O.volume(dims)
    u, psi = O.make_inputs(dims, SEED_GAUGE, SEED_SPINOR, gkind)
    ref = O.Reference(prec)
    dt = ref.np_real
    uu = np.ascontiguousarray(u.astype(dt))
    pp = np.ascontiguousarray(psi.astype(dt))
    ref.init(nd, dims, kind, lol if kind == O.LAYOUT_PERM else None)
    w = checksum_weights(V * 24)
    out = {"combos": {}, "arrays": {}}
    for isign in (1, -1):
        for cb in (0, 1):
            res = np.zeros((V, 4, 3, 2), dt)
            ref.apply(nd, uu, pp, res, isign, cb)
            r64 = res.astype(np.float64).ravel()
            key = f"{name}/f{prec}/isign{isign:+d}/cb{cb}"
            sites = sample_sites(nd, dims, lol, cb, full)
            out["combos"][key] = {"sum": float(np.dot(w, r64)), "sumsq": float(np.dot(r64, r64)),
                                  "abssum": float(np.dot(np.abs(w), np.abs(r64)))}
            out["arrays"][key + "/sites"] = sites.astype(np.int32)
            out["arrays"][key + "/values"] = res.reshape(V, 24)[sites].copy()
    if not (nd == 3 and prec == 64):
        ref.free(nd)
    return name, prec, out


def main():
    import oracle as O
    if not (O.reference_available(32) and O.reference_available(64)):
        raise SystemExit("build the reference first: make -C oracle")
    manifest = {"seeds": {"gauge": SEED_GAUGE, "spinor": SEED_SPINOR, "perm": SEED_PERM},
                "checksum": "sum = dot(w, res.ravel()), w = checksum_weights(V*24); sumsq = dot(res, res)",
                "cases": {}}
    arrays = {}
    jobs = []
    for (name, nd, dims, layout, gkind, full) in CASES:
        u, psi = O.make_inputs(dims, SEED_GAUGE, SEED_SPINOR, gkind)
        wu = checksum_weights(u.size)
        wp = checksum_weights(psi.size)
        manifest["cases"][name] = {"nd": nd, "dims": list(dims), "layout": layout, "gauge": gkind,
                                   "full": full,
                                   "input_checksums": {"u": float(np.dot(wu, u.ravel())),
                                                       "psi": float(np.dot(wp, psi.ravel()))},
                                   "combos": {}}
        for prec in (32, 64):
            jobs.append((name, nd, dims, layout, gkind, full, prec))
    ctx = mp.get_context("spawn")
    with ctx.Pool(4, maxtasksperchild=1) as pool:
        for name, prec, out in pool.imap_unordered(run_case, jobs):
            manifest["cases"][name]["combos"].update(out["combos"])
            arrays.update(out["arrays"])
    with open(os.path.join(OUT_DIR, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(OUT_DIR, "dslash_golden.npz"), **arrays)
    print("wrote", len(arrays), "arrays")


if __name__ == "__main__":
    main()
