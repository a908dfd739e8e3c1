"""Time the CPU implementations of the Dslash on one host, on the same inputs
and thread count -- TEST INFRASTRUCTURE (it pins the CPU baseline).

    python oracle/time_cpu_baselines.py [--dims 32,32,32,64] [--prec 32] [--seconds 10] [--threads N]

Times full applications (isign and cb cycled) of
* the reference library built from its own sources with the host's SSE
  (oracle/_ref/libref{32,64}.so; x86_64 hosts with the reference sources),
* the same sources built through the portable SSE shim
  (oracle/_ref/libref{32,64}_shim.so),
* the oracle's table-driven port (oracle/liboracle.so), which is the CPU
  baseline on hosts without the reference sources,
each in its own process (the reference keeps its lattice in global state),
and prints a markdown table: ms per application, GFLOP/s (1320 flop per
site) and the ratio to the reference.
"""
from __future__ import annotations

import argparse
import multiprocessing as mp
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _time(kind, prec, dims, seconds, threads, q):
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import numpy as np
    import oracle as O
    dt = np.float32 if prec == 32 else np.float64
    V = O.volume(dims)
    rng = np.random.default_rng(1234)
    u = O.random_gauge(rng, V).astype(dt)
    psi = O.gaussian_spinor(rng, V).astype(dt)
    res = np.zeros_like(psi)
    combos = [(1, 0), (-1, 1), (-1, 0), (1, 1)]
    if kind == "port":
        tabs = O.PortTables(4, dims, O.layout_table(O.LAYOUT_CB2, dims))

        def step(k):
            tabs.apply(u, psi, res, *combos[k % 4], nthreads=threads)
    else:
        R = O.Reference(prec, shim=(kind == "shim"))
        R.init(4, dims, O.LAYOUT_CB2)

        def step(k):
            R.apply(4, u, psi, res, *combos[k % 4])
    step(0)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n < 4:
        step(n + 1)
        n += 1
    q.put((time.perf_counter() - t0) / n)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", default="32,32,32,64")
    ap.add_argument("--prec", type=int, default=32)
    ap.add_argument("--seconds", type=float, default=10.0)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    a = ap.parse_args()
    dims = tuple(int(v) for v in a.dims.split(","))
    sys.path.insert(0, ROOT)
    import oracle as O
    kinds = [k for k, ok in (("reference", O.reference_available(a.prec)),
                             ("shim", O.reference_available(a.prec, shim=True)), ("port", True)) if ok]
    ctx = mp.get_context("spawn")
    out = {}
    for k in kinds:
        q = ctx.Queue()
        p = ctx.Process(target=_time, args=(k, a.prec, dims, a.seconds, a.threads, q))
        p.start()
        out[k] = q.get()
        p.join()
    sites = O.volume(dims) // 2
    print(f"host {platform.machine()}, {a.threads} threads, {'x'.join(map(str, dims))} FP{a.prec}, "
          f"full applications, isign/cb cycled, about {a.seconds:.0f} s each")
    print()
    print("| implementation | ms / application | GFLOP/s | vs reference |")
    print("|---|---|---|---|")
    names = {"reference": "reference, native SSE (oracle/_ref/libref%d.so)" % a.prec,
             "shim": "reference, portable SSE shim (oracle/_ref/libref%d_shim.so)" % a.prec,
             "port": "oracle port (oracle/liboracle.so)"}
    for k in kinds:
        ms = out[k] * 1e3
        ratio = f"{out['reference'] / out[k]:.2f}x" if "reference" in out else "-"
        print(f"| {names[k]} | {ms:.2f} | {1320 * sites / out[k] / 1e9:.1f} | {ratio} |")


if __name__ == "__main__":
    main()
