"""A plain C program built against include/sse_dslash.h and linked to the
drop-in libraries, as a C caller of the reference would be: it compiles and
links here (CPU), and on a GPU its results match the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from tests.golden_data import SITE_TOL

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SRC = os.path.join(ROOT, "tests", "c_dropin", "dslash_caller.c")
LIB = os.path.join(ROOT, "sse_wilson_dslash_gb300", "lib")


def _build(prec, out_dir):
    exe = os.path.join(out_dir, f"dslash_caller{prec}")
    cmd = ["cc", "-O2", f"-DSSE_PRECISION={prec}", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIB, f"-lgbdslash{prec}", f"-Wl,-rpath,{LIB}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("prec", [32, 64])
def test_c_caller_compiles_and_links(prec, tmp_path):
    if not os.path.exists(os.path.join(LIB, f"libgbdslash{prec}.so")):
        pytest.skip("libraries not built")
    assert os.path.exists(_build(prec, str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [32, 64])
def test_c_caller_matches_oracle(prec, tmp_path):
    dims = (8, 4, 6, 4)
    exe = _build(prec, str(tmp_path))
    out = str(tmp_path / "out.bin")
    subprocess.run([exe, *map(str, dims), out], check=True, timeout=120)
    V = O.volume(dims)
    dt = np.float32 if prec == 32 else np.float64
    raw = np.fromfile(out, dtype=dt)
    u = raw[:V * 72].astype(np.float64)
    psi = raw[V * 72:V * 96].astype(np.float64)
    res = raw[V * 96:].reshape(4, V * 24)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    k = 0
    for isign in (1, -1):
        for cb in (0, 1):
            ref = O.dslash_plain(4, dims, lol, u, psi, isign, cb)
            ts = O.target_sites(4, dims, lol, cb)
            assert O.site_rel_err(res[k], ref, ts) <= SITE_TOL[prec], (isign, cb)
            # sites of checkerboard cb are not written (the output was zeroed)
            other = np.setdiff1d(np.arange(V), ts)
            assert np.all(res[k].reshape(V, 24)[other] == 0)
            k += 1
