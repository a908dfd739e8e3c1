"""Loader for the golden vectors in tests/golden (made by make_golden.py)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def checksum_weights(n: int) -> np.ndarray:
    k = np.arange(n, dtype=np.uint64)
    h = (k * np.uint64(2654435761) + np.uint64(12345)) % np.uint64(2 ** 32)
    return h.astype(np.float64) / 2.0 ** 32 - 0.5


def load():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        man = json.load(f)
    arr = np.load(os.path.join(GOLDEN, "dslash_golden.npz"))
    return man, arr


def layout(case, dims):
    import oracle as O
    name = case["layout"]
    if name == "cb2":
        return O.LAYOUT_CB2, O.layout_table(O.LAYOUT_CB2, dims)
    if name == "cb3d":
        return O.LAYOUT_CB3D, O.layout_table(O.LAYOUT_CB3D, dims)
    if name == "lex":
        return O.LAYOUT_LEX, O.layout_table(O.LAYOUT_LEX, dims)
    return O.LAYOUT_PERM, O.scrambled_table(dims, 7)


# Tolerances (per site: ||got - ref|| / ||ref||; checksums relative to abssum)
SITE_TOL = {32: 1e-6, 64: 1e-13}
SUM_TOL = {32: 1e-6, 64: 1e-13}


def check_against_golden(man, arr, name, prec, isign, cb, res):
    """Assert res (caller-order output, full lattice) matches the golden entry."""
    key = f"{name}/f{prec}/isign{isign:+d}/cb{cb}"
    g = man["cases"][name]["combos"][key]
    r = np.asarray(res, dtype=np.float64).ravel()
    w = checksum_weights(r.size)
    s = float(np.dot(w, r))
    assert abs(s - g["sum"]) <= SUM_TOL[prec] * g["abssum"], (key, s, g["sum"])
    ss = float(np.dot(r, r))
    assert abs(ss - g["sumsq"]) <= 2 * SUM_TOL[prec] * g["sumsq"], (key, ss, g["sumsq"])
    sites = arr[key + "/sites"]
    vals = arr[key + "/values"].astype(np.float64)
    got = r.reshape(-1, 24)[sites]
    err = np.sqrt(((got - vals) ** 2).sum(1)) / np.sqrt((vals ** 2).sum(1))
    assert err.max() <= SITE_TOL[prec], (key, err.max())
    return float(err.max())
