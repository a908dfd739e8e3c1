#!/usr/bin/env python
"""Wilson Dslash benchmark: 4D, 32^3x64, FP32, 18-real links (the reference ABI).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one application of the hopping term to one checkerboard
(1,048,576 output sites), cycling isign = +1/-1 and cb = 0/1.  Prints ONE JSON
line on rank 0:

  value       GFLOP/s of the device-resident kernel (1320 flop/site), inputs
              resident in HBM; the gauge field (576 MiB) and spinors (2 x 96 MiB)
              exceed the 129 MB L2, so no flush is needed between steps
  e2e         the same metric through the drop-in C ABI (sse_su3dslash_wilson
              of libgbdslash32.so) on pinned host arrays: host->device copy of
              u and psi, the kernels and the device->host copy of res, every step
  roofline    HBM bytes of the Dslash kernel (768 B/site compulsory) per launch
              over its CUDA-event time, against MEASURED_PEAKS.json
  cpu_baseline the oracle's table-driven port (OpenMP) on the host cores, on a
              bounded slice of the same workload
  variants    recon-12, FP64 (native and in double-float arithmetic), the 3D
              operator on 24^3x48, several right-hand sides on 24^3x48, the
              uneven batch, the force, one rank's slab of the lattice split
              along t (not the headline)

--impl reference times the CPU implementation of the path on the host cores:
the reference library built from its own sources (oracle/_ref) where it was
built for this host, else the oracle's port of it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DIMS = (32, 32, 32, 64)
DIMS_3D = (24, 24, 24, 48)
FLOPS_4D, FLOPS_3D = 1320, 984
WORKLOAD = "wilson_dslash_4d_32x32x32x64_f32_recon18"
METRIC = "Dslash GFLOP/s at 32^3x64 (FP32, 4D, 18-real links, 1320 flop/site)"
DATA = "synthetic: random SU(3) links (Gaussian, Gram-Schmidt, row2 = conj(row0 x row1)), N(0,1) spinors"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def headline_config(sites):
    """The workload description both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "lattice": list(DIMS), "nd": 4, "prec": 32, "recon": 18,
            "sites_per_step": sites, "flops_per_site": FLOPS_4D, "bytes_per_site": 2 * 96 + 8 * 72,
            "l2": "no flush: inputs (gauge %d MiB, spinors 2 x %d MiB) exceed the 129 MB L2"
                  % (2 * sites * 4 * 72 >> 20, sites * 96 >> 20)}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_time_max(ms_total, world, device):
    """The slowest rank's timed-region duration: each rank runs one replica of
    the same workload, so the job takes as long as its slowest replica."""
    if world <= 1:
        return ms_total
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_total], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gflops(ms_total, world, sites, steps):
    """Whole-job GFLOP/s: all replicas' output sites over the slowest time."""
    return FLOPS_4D * sites * steps * world / (ms_total * 1e6)


# ---------------------------------------------------------------------------
# Clock sampling (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.marks = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception as e:  # no nvidia-smi: report without clocks
            log("clock sampler unavailable:", e)
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.time(), ln.strip()))

    def mark(self, what):
        self.marks.append((what, time.time()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, ln in self.lines:
            if not (t0 - 0.15 <= ts <= t1 + 0.15):
                continue
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# Synthetic inputs on the device (random SU(3) links, N(0,1) spinors)
# ---------------------------------------------------------------------------

def su3_links(n, gen, torch):
    """n random SU(3) matrices: Gaussian complex rows, Gram-Schmidt, row 2 =
    conj(row0 x row1); returned packed as [n][j][i][2] (transposed), float64."""
    out = torch.empty(n, 3, 3, 2, dtype=torch.float64, device="cuda")
    chunk = 1 << 22
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        g = torch.randn(m, 2, 3, 2, dtype=torch.float64, device="cuda", generator=gen)
        a = torch.view_as_complex(g)
        r0 = a[:, 0] / a[:, 0].abs().pow(2).sum(-1, keepdim=True).sqrt()
        r1 = a[:, 1] - (r0.conj() * a[:, 1]).sum(-1, keepdim=True) * r0
        r1 = r1 / r1.abs().pow(2).sum(-1, keepdim=True).sqrt()
        r2 = torch.linalg.cross(r0, r1).conj()
        U = torch.stack([r0, r1, r2], dim=1)              # U[i][j]
        out[s:s + m] = torch.view_as_real(U.transpose(1, 2).contiguous())  # [j][i]
    return out


def near_unit_links(n, gen, torch, eps=0.3):
    """n matrices exp(i*eps*H), H traceless Hermitian with N(0,1) entries,
    packed [n][j][i][2] (transposed), float64."""
    out = torch.empty(n, 3, 3, 2, dtype=torch.float64, device="cuda")
    chunk = 1 << 21
    iu = torch.triu_indices(3, 3, 1, device="cuda")
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        d = torch.randn(m, 3, dtype=torch.float64, device="cuda", generator=gen)
        od = torch.randn(m, 3, 2, dtype=torch.float64, device="cuda", generator=gen)
        H = torch.zeros(m, 3, 3, dtype=torch.complex128, device="cuda")
        H.diagonal(dim1=1, dim2=2).copy_((d - d.mean(1, keepdim=True)).to(torch.complex128))
        off = torch.view_as_complex(od)
        H[:, iu[0], iu[1]] = off
        H[:, iu[1], iu[0]] = off.conj()
        U = torch.linalg.matrix_exp(1j * eps * H)
        out[s:s + m] = torch.view_as_real(U.transpose(1, 2).contiguous())
    return out


def run_solver_bench(torch, log_fn):
    """Time to |c - A x| <= 1e-10 |c| for the even-odd Wilson operator,
    kappa = 0.124, 32^3x64, near-unit links: all-FP64 CG vs FP32 CG inside FP64
    defect correction."""
    from sse_wilson_dslash_gb300.device import WilsonSolver
    dims = (32, 32, 32, 64)
    V = dims[0] * dims[1] * dims[2] * dims[3]
    gen = torch.Generator(device="cuda").manual_seed(99)
    u = near_unit_links(V * 4, gen, torch).reshape(-1)
    b = torch.randn(V * 24, dtype=torch.float64, device="cuda", generator=gen)
    out = {"lattice": list(dims), "kappa": 0.124, "links": "exp(i 0.3 H), H traceless Hermitian N(0,1)",
           "source": "N(0,1)", "tol": 1e-10, "residual": "|M^+ b - M^+ M x| / |M^+ b| (CG on M^+ M)"}
    sols = {}
    # *_fp64: the outer residual on the FP64 operator (the default);
    # *_df_outer: on the operator in double-float arithmetic (FP32 pipes)
    for name, prec, recon, itol, dfo in (("fp64_cg", 64, 18, 1e-5, False), ("mixed_fp32_fp64", 32, 12, 1e-5, False),
                                         ("mixed_fp16_fp64", 16, 12, 1e-3, False),
                                         ("mixed_bf16_fp64", 17, 12, 1e-3, False),
                                         ("mixed_fp32_df_outer", 32, 12, 1e-5, True),
                                         ("mixed_fp16_df_outer", 16, 12, 1e-3, True)):
        s = WilsonSolver(dims, 0.124, tol=1e-10, max_iter=20000, inner_prec=prec, inner_recon=recon, inner_tol=itol,
                         outer_double_float=dfo)
        s.set_gauge(u)
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = s.solve(b, x)
        torch.cuda.synchronize()
        st["wall_seconds"] = time.perf_counter() - t0
        st["inner_recon"] = recon
        out[name] = st
        sols[name] = x
        log_fn(name, st)
        s.close()
        del s
        torch.cuda.empty_cache()
    out["speedup"] = out["fp64_cg"]["wall_seconds"] / out["mixed_fp32_fp64"]["wall_seconds"]
    for k in ("mixed_fp32_fp64", "mixed_fp16_fp64", "mixed_bf16_fp64", "mixed_fp32_df_outer", "mixed_fp16_df_outer"):
        out[k]["speedup_vs_fp64"] = out["fp64_cg"]["wall_seconds"] / out[k]["wall_seconds"]
        out[k]["solution_rel_diff"] = float((sols["fp64_cg"] - sols[k]).norm() / sols["fp64_cg"].norm())
    # batched: 16 right-hand sides (the first is the source above), FP32
    # inner CGs in lockstep on the multi-RHS operator, FP64 defect correction
    from sse_wilson_dslash_gb300.device import BatchedWilsonSolver
    nrhs = 16
    bb = torch.randn(nrhs, V * 24, dtype=torch.float64, device="cuda", generator=gen)
    bb[0] = b
    del sols
    torch.cuda.empty_cache()
    for name, dfo, single, key in (("batched_fp32_fp64_nrhs16", False, "mixed_fp32_fp64", "mixed_fp32"),
                                   ("batched_fp32_df_outer_nrhs16", True, "mixed_fp32_df_outer", "mixed_fp32_df_outer")):
        bs = BatchedWilsonSolver(dims, nrhs, 0.124, tol=1e-10, max_iter=20000, inner_recon=12, outer_double_float=dfo)
        bs.set_gauge(u)
        xx = torch.zeros_like(bb)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sts = bs.solve(bb, xx)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        per_rhs = wall / nrhs
        out[name] = {
            "nrhs": nrhs, "wall_seconds": wall, "seconds_per_rhs": per_rhs,
            "iterations_max": max(t["iterations"] for t in sts), "cycles_max": max(t["cycles"] for t in sts),
            "converged": int(all(t["converged"] for t in sts)), "residual_max": max(t["residual"] for t in sts),
            "true_residual_max": max(t["true_residual"] for t in sts),
            "speedup_per_rhs_vs_fp64": out["fp64_cg"]["wall_seconds"] / per_rhs,
            f"speedup_per_rhs_vs_{key}": out[single]["wall_seconds"] / per_rhs}
        log_fn(name, out[name])
        bs.close()
        del bs, xx
        torch.cuda.empty_cache()
    del bb
    torch.cuda.empty_cache()
    return out


def make_fields(dims, dtype, torch, seed=1234):
    V = dims[0] * dims[1] * dims[2] * dims[3]
    gen = torch.Generator(device="cuda").manual_seed(seed)
    u = su3_links(V * 4, gen, torch).to(dtype).reshape(-1)
    psi = torch.randn(V * 24, dtype=dtype, device="cuda", generator=gen)
    return u, psi


# ---------------------------------------------------------------------------
# Timing helpers
# ---------------------------------------------------------------------------

def time_device(op, gauge, srcs, outs, steps, warmup, torch):
    """Average ms per Dslash launch, CUDA events on the launching stream."""
    stream = torch.cuda.current_stream()
    combos = [(1, 0), (-1, 1), (-1, 0), (1, 1)]
    for k in range(warmup):
        isign, cb = combos[k % 4]
        op.apply(gauge, srcs[cb], isign, cb, out=outs[1 - cb], stream=stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(steps):
        isign, cb = combos[k % 4]
        op.apply(gauge, srcs[cb], isign, cb, out=outs[1 - cb], stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def device_variant(dims, nd, prec, recon, steps, warmup, torch, fields=None, fmt="native"):
    from sse_wilson_dslash_gb300.device import DslashOperator
    op = DslashOperator(dims, nd=nd, prec=prec, recon=recon, spinor_format=fmt)
    dt = torch.float32 if prec == 32 else torch.float64
    u, psi = fields if fields is not None else make_fields(dims, dt, torch)
    gauge = op.pack_gauge(u)
    srcs = [op.pack_spinor(psi, 0), op.pack_spinor(psi, 1)]
    outs = [op.new_spinor(), op.new_spinor()]
    tuning = op.autotune(gauge, srcs[0], outs[1])
    ms = time_device(op, gauge, srcs, outs, steps, warmup, torch)
    sites = op.volume_cb
    res = {"ms": ms, "gflops": op.flops_per_site * sites / (ms * 1e6),
           "gbs": op.bytes_per_site * sites / (ms * 1e6), "bytes_per_site": op.bytes_per_site,
           "flops_per_site": op.flops_per_site, "sites": sites, "tuning": list(tuning)}
    del gauge, srcs, outs
    op.close()
    return res


def multi_rhs_variants(torch, steps, peak):
    """Several right-hand sides on one 24^3x48 gauge field: FP32, FP32 in
    spin pairs and BF16 spinor storage, 18-real links; GFLOP/s counts 1320
    flop per site and right-hand side."""
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (24, 24, 24, 48)
    V = dims[0] * dims[1] * dims[2] * dims[3]
    gen = torch.Generator(device="cuda").manual_seed(7)
    u = su3_links(V * 4, gen, torch).float().reshape(-1)
    out = {}
    names = {"native": "f32", "f32_pairs": "f32pairs", "bf16": "bf16"}
    for fmt, counts in (("native", (1, 4, 8, 16, 32)), ("f32_pairs", (16, 32)), ("bf16", (1, 4, 8, 16, 32))):
        for nrhs in counts:
            op = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
            gauge = op.pack_gauge(u)
            psi = torch.randn(nrhs * V * 24, dtype=torch.float32, device="cuda", generator=gen)
            srcs = [op.pack_spinor(psi, 0), op.pack_spinor(psi, 1)]
            del psi
            outs = [op.new_spinor(), op.new_spinor()]
            ms = time_device(op, gauge, srcs, outs, max(10, steps // max(1, nrhs // 4)), 3, torch)
            sites = op.volume_cb * nrhs
            gbs = op.bytes_per_site * sites / (ms * 1e6)
            out[f"{names[fmt]}_nrhs{nrhs}"] = {
                "ms": ms, "gflops": 1320 * sites / (ms * 1e6), "gbs": gbs, "roofline_frac": gbs / peak,
                "ms_per_rhs": ms / nrhs, "bytes_per_site_rhs": op.bytes_per_site, "variant": op.tuning()[1]}
            del gauge, srcs, outs
            op.close()
            torch.cuda.empty_cache()
    # 16-bit storage with 16 / 32 right-hand sides: colour multiply on the
    # CUDA cores ("cc") and on the tensor cores ("tc")
    for fmt in ("bf16", "f16"):
        for nrhs in (16, 32):
            for tc in (False, True):
                key = f"{fmt}_nrhs{nrhs}_{'tc' if tc else 'cc'}"
                if not tc and fmt == "bf16":
                    out[key] = out[f"bf16_nrhs{nrhs}"]
                    continue
                op = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs, spinor_format=fmt)
                if tc:
                    op.set_tensor_cores(True)
                gauge = op.pack_gauge(u)
                psi = torch.randn(nrhs * V * 24, dtype=torch.float32, device="cuda", generator=gen)
                srcs = [op.pack_spinor(psi, 0), op.pack_spinor(psi, 1)]
                del psi
                outs = [op.new_spinor(), op.new_spinor()]
                ms = time_device(op, gauge, srcs, outs, max(10, steps // max(1, nrhs // 4)), 3, torch)
                op.check()
                sites = op.volume_cb * nrhs
                gbs = op.bytes_per_site * sites / (ms * 1e6)
                out[key] = {"ms": ms, "gflops": 1320 * sites / (ms * 1e6), "gbs": gbs, "roofline_frac": gbs / peak,
                            "ms_per_rhs": ms / nrhs, "bytes_per_site_rhs": op.bytes_per_site,
                            "variant": "tc" if tc else op.tuning()[1]}
                del gauge, srcs, outs
                op.close()
                torch.cuda.empty_cache()
    return out


def uneven_batch(torch, peak):
    """16^4 (8 rhs), 20^3x40 (4), 24^3x48 (2), 32^3x64 (1), each with its own
    random SU(3) gauge field: four separate launches vs one persistent launch
    (autotuned schedule) vs the same launch replayed from a CUDA graph."""
    from sse_wilson_dslash_gb300.device import DslashBatch, DslashOperator
    specs = [((16, 16, 16, 16), 8), ((20, 20, 20, 40), 4), ((24, 24, 24, 48), 2), ((32, 32, 32, 64), 1)]
    gen = torch.Generator(device="cuda").manual_seed(11)
    items = []
    for dims, nrhs in specs:
        op = DslashOperator(dims, nd=4, prec=32, recon=18, nrhs=nrhs)
        V = op.volume
        u = su3_links(V * 4, gen, torch).float().reshape(-1)
        gauge = op.pack_gauge(u)
        del u
        psi = torch.randn(nrhs * V * 24, dtype=torch.float32, device="cuda", generator=gen)
        items.append(dict(op=op, gauge=gauge, psi=op.pack_spinor(psi, 0), res=op.new_spinor(), isign=1, cb=0))
        del psi
    work = sum(1320 * it["op"].volume_cb * it["op"].nrhs for it in items)
    nbytes = sum(it["op"].bytes_per_site * it["op"].volume_cb * it["op"].nrhs for it in items)
    stream = torch.cuda.Stream()
    reps = 50

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(3):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / reps

    def separate():
        for it in items:
            it["op"].apply(it["gauge"], it["psi"], 1, 0, out=it["res"], stream=stream)

    ms_sep = timed(separate)
    b = DslashBatch(items)
    with torch.cuda.stream(stream):
        sched = b.autotune(stream)
    ms_one = timed(lambda: b.launch(stream))
    with torch.cuda.stream(stream):
        b.capture_graph(stream)
    ms_graph = timed(lambda: b.launch(stream))
    b.close()
    out = {"lattices": [dict(dims=list(d), nrhs=n) for d, n in specs], "schedule": sched,
           "separate_ms": ms_sep, "one_launch_ms": ms_one, "graph_ms": ms_graph,
           "gflops_graph": work / (ms_graph * 1e6), "gbs_graph": nbytes / (ms_graph * 1e6),
           "roofline_frac_graph": nbytes / (ms_graph * 1e6) / peak}
    for it in items:
        it["op"].close()
    return out


def force_variants(torch, peak, steps):
    """dL/dU of L = Re <chi, D psi> for every link (gbds_op_force, mode 1: the
    su(3) force TA(G U^+), written in the packed gauge layout), at the
    configured sizes: 32^3x64 in FP32 and 16^4 in FP64.  Algorithmic bytes per
    call: the V/2 source spinors and V/2 chi spinors read once, the 4 links
    of each site read once and their forces written once: V (s + 8 g), s and
    g the bytes of a spinor and of a link.  Each call is timed alone with CUDA
    events, after writing a 256 MiB buffer so that no input is left in L2 (the
    16^4 fields would fit in it)."""
    from sse_wilson_dslash_gb300.device import DslashOperator
    out = {}
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    for dims, prec in (((32, 32, 32, 64), 32), ((16, 16, 16, 16), 64)):
        dt = torch.float32 if prec == 32 else torch.float64
        op = DslashOperator(dims, nd=4, prec=prec, recon=18)
        V = op.volume
        u, psi = make_fields(dims, dt, torch, seed=21)
        gen = torch.Generator(device="cuda").manual_seed(22)
        chi = torch.randn(V * 24, dtype=dt, device="cuda", generator=gen)
        gauge = op.pack_gauge(u)
        srcs = {cb: (op.pack_spinor(psi, cb), op.pack_spinor(chi, 1 - cb)) for cb in (0, 1)}
        del u, psi, chi
        f = torch.empty(V * 72, dtype=dt, device="cuda")
        combos = [(1, 0), (-1, 1), (-1, 0), (1, 1)]
        stream = torch.cuda.current_stream()
        for k in range(3):
            isign, cb = combos[k % 4]
            op.force(gauge, srcs[cb][0], srcs[cb][1], isign, cb, f, mode=1, stream=stream)
        n = max(10, min(steps, 50))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for k in range(n):
            isign, cb = combos[k % 4]
            flush.fill_(float(k))
            ev[k][0].record(stream)
            op.force(gauge, srcs[cb][0], srcs[cb][1], isign, cb, f, mode=1, stream=stream)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / n
        real = 4 if prec == 32 else 8
        nbytes = V * (24 * real + 8 * 18 * real)
        gbs = nbytes / (ms * 1e6)
        out["force_%s_f%d" % ("x".join(map(str, dims)), prec)] = {
            "ms": ms, "gbs": gbs, "roofline_frac": gbs / peak, "bytes_per_call": nbytes,
            "links": 4 * V, "launches_per_call": 1, "mode": "su(3) force TA(G U^+)"}
        del gauge, srcs, f
        op.close()
        torch.cuda.empty_cache()
    del flush
    return out


def split_t_variant(torch, peak, steps):
    """One rank's slab when 32^3x64 is split along t across two GPUs: the
    32^3x32 slab's periodic Dslash against the split form (pack the two send
    faces, move them -- here a device copy stands in for the transfer between
    GPUs --, the interior time slices, then the two boundary slices), FP32,
    18-real links, CUDA events over `steps` applications of each."""
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (32, 32, 32, 32)
    op = DslashOperator(dims, nd=4, prec=32, recon=18)
    u, psi = make_fields(dims, torch.float32, torch, seed=31)
    gauge = op.pack_gauge(u)
    src = op.pack_spinor(psi, 0)
    del u, psi
    out = op.new_spinor()
    faces = [op.new_face() for _ in range(4)]
    stream = torch.cuda.current_stream()

    def periodic():
        op.apply(gauge, src, 1, 0, out=out, stream=stream)

    def split():
        op.pack_faces(gauge, src, 1, 0, faces[0], faces[1], stream=stream)
        faces[3].copy_(faces[0])
        faces[2].copy_(faces[1])
        op.apply_halo(gauge, src, None, None, 1, 0, out=out, part="interior", stream=stream)
        op.apply_halo(gauge, src, faces[2], faces[3], 1, 0, out=out, part="boundary", stream=stream)

    def timed(fn, n):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    n = max(20, min(steps, 200))
    ms_p = timed(periodic, n)
    ms_s = timed(split, n)
    ms_pack = timed(lambda: op.pack_faces(gauge, src, 1, 0, faces[0], faces[1], stream=stream), n)
    sites = op.volume_cb
    res = {"slab": list(dims), "of_lattice": [32, 32, 32, 64], "ranks": 2,
           "periodic_ms": ms_p, "split_ms": ms_s, "pack_faces_ms": ms_pack,
           "split_gflops": 1320 * sites / (ms_s * 1e6),
           "split_roofline_frac": op.bytes_per_site * sites / (ms_s * 1e6) / peak,
           "face_bytes": op.face_bytes, "faces_per_rank_per_application": 2}
    del gauge, src, out, faces
    op.close()
    torch.cuda.empty_cache()
    return res


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload):
    """Per-launch DRAM bytes of the Dslash kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"{workload}.md")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.strip().startswith("traffic_bytes_per_launch:"):
            # measured for one launch by ncu (dram__bytes_read.sum + dram__bytes_write.sum)
            try:
                return int(float(ln.split(":", 1)[1].strip()))
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------------------
# CPU legs
# ---------------------------------------------------------------------------

def cpu_stepper(u_host, psi_host):
    """One full application of the CPU implementation of the path on the
    host cores, as step(k) cycling isign/cb: the reference library built from
    its own sources (oracle/_ref) where it exists for this host, else the
    oracle's table-driven port of it.  Returns (step, kind, threads, what)."""
    import numpy as np
    import oracle as O
    res = np.zeros_like(psi_host)
    combos = [(1, 0), (-1, 1), (-1, 0), (1, 1)]
    threads = O.max_threads()
    if O.reference_available(32):
        try:
            ref = O.Reference(32)
            ref.init(4, DIMS, O.LAYOUT_CB2)

            def step(k):
                isign, cb = combos[k % 4]
                ref.apply(4, u_host, psi_host, res, isign, cb)
            return step, "reference", threads, ("sse_su3dslash_wilson of the reference library built from its own "
                                                 "sources (OpenMP dispatch)")
        except OSError:
            pass
    tabs = O.PortTables(4, DIMS, O.layout_table(O.LAYOUT_CB2, DIMS))

    def step(k):
        isign, cb = combos[k % 4]
        tabs.apply(u_host, psi_host, res, isign, cb, threads)
    return step, "port", threads, ("the oracle's table-driven port of the reference scalar library (OpenMP); "
                                   "the reference sources are not on this host")


def cpu_rate(u_host, psi_host, seconds):
    """GFLOP/s of full applications of the CPU implementation for about
    ``seconds`` (after one untimed application)."""
    step, kind, threads, what = cpu_stepper(u_host, psi_host)
    Vh = u_host.shape[0] // 2
    step(0)
    apps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        step(apps + 1)
        apps += 1
    dt = time.perf_counter() - t0
    return FLOPS_4D * Vh * apps / dt / 1e9, kind, threads, apps, dt, what


def run_reference(args):
    """--impl reference: the CPU implementation of the path on the host cores."""
    import numpy as np
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    V = O.volume(DIMS)
    Vh = V // 2
    rng = np.random.default_rng(1234)
    log("reference arm: generating inputs")
    u = O.random_gauge(rng, V).astype(np.float32)
    psi = O.gaussian_spinor(rng, V).astype(np.float32)
    step, kind, threads, what = cpu_stepper(u, psi)
    sample = f"full {'x'.join(map(str, DIMS))} FP32 applications, isign/cb cycled: " + what
    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(args.steps):
        step(k)
    dt = time.perf_counter() - t0
    value = FLOPS_4D * Vh * args.steps / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": DATA, "config": headline_config(Vh),
            "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------

def run_gb300(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    from sse_wilson_dslash_gb300 import _lib
    from sse_wilson_dslash_gb300.device import DslashOperator
    from sse_wilson_dslash_gb300.legacy import SSEDslash

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # -- the headline: device-resident FP32 4D 32^3x64 recon 18 --------------
    op = DslashOperator(DIMS, nd=4, prec=32, recon=18)
    u, psi = make_fields(DIMS, torch.float32, torch)
    gauge = op.pack_gauge(u)
    srcs = [op.pack_spinor(psi, 0), op.pack_spinor(psi, 1)]
    outs = [op.new_spinor(), op.new_spinor()]
    if args.tuning:
        blk, var = (int(v) for v in args.tuning.split(","))
        op.set_tuning(blk, var)
        tuning = op.tuning()
    else:
        tuning = op.autotune(gauge, srcs[0], outs[1])
    stream = torch.cuda.current_stream()
    combos = [(1, 0), (-1, 1), (-1, 0), (1, 1)]
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    gpu_index = int(vis.split(",")[local]) if vis and vis.split(",")[local].strip().isdigit() else local
    clocks = ClockSampler(gpu_index)
    clocks.start()
    time.sleep(0.3)
    for k in range(args.warmup):
        isign, cb = combos[k % 4]
        op.apply(gauge, srcs[cb], isign, cb, out=outs[1 - cb], stream=stream)
    barrier()
    launches0 = _lib.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall0 = time.time()
    e0.record(stream)
    for k in range(args.steps):
        isign, cb = combos[k % 4]
        op.apply(gauge, srcs[cb], isign, cb, out=outs[1 - cb], stream=stream)
    e1.record(stream)
    barrier()
    t_wall1 = time.time()
    launches = _lib.launch_count() - launches0
    ms_total = replica_time_max(e0.elapsed_time(e1), world, "cuda")
    ms = ms_total / args.steps
    sites = op.volume_cb
    value = replica_gflops(ms_total, world, sites, args.steps)
    bytes_per_site = op.bytes_per_site
    achieved = bytes_per_site * sites / (ms * 1e6)
    # Keep the clock sampler running a little longer to cover short regions.
    extra = time.time()
    while time.time() - extra < 0.5:
        for k in range(200):
            isign, cb = combos[k % 4]
            op.apply(gauge, srcs[cb], isign, cb, out=outs[1 - cb], stream=stream)
        torch.cuda.synchronize()
    t_wall1b = time.time()
    clk = clocks.summary(t_wall0, t_wall1b)
    clocks.stop()

    peak, peak_kind = load_peaks()
    traffic = profiled_traffic(WORKLOAD)

    # -- e2e through the drop-in C ABI on pinned host memory ----------------
    e2e = None
    cpu = None
    if not args.no_e2e:  # every rank: replicas
        u_h = torch.empty(u.numel(), dtype=torch.float32, pin_memory=True)
        u_h.copy_(u.cpu())
        psi_h = torch.empty(psi.numel(), dtype=torch.float32, pin_memory=True)
        psi_h.copy_(psi.cpu())
        res_h = torch.zeros(psi.numel(), dtype=torch.float32, pin_memory=True)
        del gauge, srcs, outs
        torch.cuda.empty_cache()
        d = SSEDslash(32)
        d.init_sse_su3dslash(DIMS, *_lib.canonical_callbacks(4, DIMS))
        e2e_steps = max(5, min(args.steps, 50))
        for k in range(max(2, min(args.warmup, 5))):
            isign, cb = combos[k % 4]
            d.sse_su3dslash_wilson(u_h, psi_h, res_h, isign, cb)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            isign, cb = combos[k % 4]
            d.sse_su3dslash_wilson(u_h, psi_h, res_h, isign, cb)
        torch.cuda.synchronize()
        barrier()
        dt = time.perf_counter() - t0
        from sse_wilson_dslash_gb300 import legacy
        path = "direct (kernels read/write the pinned host arrays over NVLink-C2C)" if legacy.last_path() == 1 \
            else "staged (cudaMemcpyAsync)"
        e2e = {"value": FLOPS_4D * sites * e2e_steps * world / dt / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": op.volume * 72 * 4 + sites * 96, "d2h_bytes_per_step": sites * 96,
               "steps": e2e_steps, "ms_per_step": dt / e2e_steps * 1e3,
               "path": "sse_su3dslash_wilson (libgbdslash32.so), pinned host arrays, gauge read every call, "
                       + path}
        # the same calls staged through cudaMemcpyAsync, for comparison
        legacy.set_host_access(1)
        d.sse_su3dslash_wilson(u_h, psi_h, res_h, 1, 0)
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            isign, cb = combos[k % 4]
            d.sse_su3dslash_wilson(u_h, psi_h, res_h, isign, cb)
        dt_s = time.perf_counter() - t0
        legacy.set_host_access(0)
        e2e["staged"] = {"value": FLOPS_4D * sites * e2e_steps * world / dt_s / 1e9, "ms_per_step": dt_s / e2e_steps * 1e3}
        # gauge-resident variant: the caller promises u is unchanged between calls
        legacy.set_gauge_cache(True)
        d.sse_su3dslash_wilson(u_h, psi_h, res_h, 1, 0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            isign, cb = combos[k % 4]
            d.sse_su3dslash_wilson(u_h, psi_h, res_h, isign, cb)
        dt = time.perf_counter() - t0
        legacy.set_gauge_cache(False)
        e2e["gauge_resident"] = {"value": FLOPS_4D * sites * e2e_steps * world / dt / 1e9,
                                 "ms_per_step": dt / e2e_steps * 1e3,
                                 "h2d_bytes_per_step": sites * 96, "d2h_bytes_per_step": sites * 96}
        d.free_sse_su3dslash()
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            uh = u_h.numpy().reshape(-1, 4, 3, 3, 2)
            ph = psi_h.numpy().reshape(-1, 4, 3, 2)
            rate, kind, n, apps, secs, what = cpu_rate(uh, ph, args.cpu_seconds)
            cpu = {"value": rate, "unit": "GFLOP/s", "cores": n, "kind": kind,
                   "sample": f"{apps} full {'x'.join(map(str, DIMS))} FP32 applications in {secs:.1f} s, isign/cb "
                             f"cycled, on the same inputs as the GPU: " + what}
        del u_h, psi_h, res_h

    # -- variants (not the headline) -------------------------------------------
    variants = {}
    if not args.no_variants:
        vsteps = max(20, min(args.steps, 200))
        want = set(args.variants.split(","))
        run = lambda name: "all" in want or name in want  # noqa: E731
        if run("recon12"):
            variants["f32_recon12"] = device_variant(DIMS, 4, 32, 12, vsteps, 5, torch, fields=(u, psi))
        if run("f64"):
            u64, psi64 = u.double(), psi.double()
            del u, psi
            torch.cuda.empty_cache()
            variants["f64_recon18"] = device_variant(DIMS, 4, 64, 18, vsteps, 5, torch, fields=(u64, psi64))
            variants["f64_recon12"] = device_variant(DIMS, 4, 64, 12, vsteps, 5, torch, fields=(u64, psi64))
            # the FP64 operator in double-float arithmetic on the FP32 pipes
            # (FP64-sized fields, ~48 significant bits)
            variants["f64_double_float_recon18"] = device_variant(DIMS, 4, 64, 18, vsteps, 5, torch,
                                                                  fields=(u64, psi64), fmt="double_float")
            del u64, psi64
        else:
            del u, psi
        torch.cuda.empty_cache()
        if run("3d"):
            variants["3d_24x24x24x48_f32_recon18"] = device_variant(DIMS_3D, 3, 32, 18, vsteps, 5, torch)
            variants["3d_24x24x24x48_f32_recon12"] = device_variant(DIMS_3D, 3, 32, 12, vsteps, 5, torch)
        for v in variants.values():
            v["roofline_frac"] = v["gbs"] / peak
        if run("multi_rhs"):
            variants["multi_rhs_24x24x24x48"] = multi_rhs_variants(torch, vsteps, peak)
            torch.cuda.empty_cache()
        if run("uneven_batch"):
            variants["uneven_batch"] = uneven_batch(torch, peak)
        if run("force"):
            variants.update(force_variants(torch, peak, vsteps))
        if run("split_t"):
            variants["split_t_32x32x32x64_2ranks_f32"] = split_t_variant(torch, peak, vsteps)

    solver = None
    if not args.no_solver:
        torch.cuda.empty_cache()
        solver = run_solver_bench(torch, log)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": DATA, "config": headline_config(sites),
                "parallelism": "replicas" if world > 1 else "single GPU",
                "tuning": {"block": tuning[0], "variant": tuning[1]},
                "hbm_gbs": achieved,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_source": peak_kind,
                             "traffic": traffic, "algorithmic_bytes_per_launch": bytes_per_site * sites,
                             "kernel": "gbds::dslash_kernel<float,4,18,isign>"},
                "gflops_ref_convention": 1390 * sites / (ms * 1e6),
                "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
                "variants": variants, "solver": solver}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """--profile KIND: build one operator on --dims and launch only its kernel,
    --warmup + --steps times, for an ncu capture (-k, -s, -c select the
    launches).  KIND: dslash (--prec, --recon), force (--prec; the su(3)
    force), multi_rhs (--nrhs, --fmt, --variant or --tc).  Prints one JSON
    line with the mean CUDA-event time of the timed launches; nothing else is
    allocated beyond the operator's fields."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = DIMS
    V = dims[0] * dims[1] * dims[2] * dims[3]
    gen = torch.Generator(device="cuda").manual_seed(5)
    kind = args.profile
    if kind == "multi_rhs":
        op = DslashOperator(dims, nd=4, prec=32, recon=args.recon, nrhs=args.nrhs, spinor_format=args.fmt)
        if args.tc:
            op.set_tensor_cores(True)
        elif args.variant >= 0:
            op.set_tuning(0, args.variant)
        op.set_site_order(args.zblock)
        u = su3_links(V * 4, gen, torch).float().reshape(-1)
        psi = torch.randn(args.nrhs * V * 24, dtype=torch.float32, device="cuda", generator=gen)
    else:
        dt = torch.float32 if args.prec == 32 else torch.float64
        fmt = "double_float" if (kind == "dslash" and args.fmt == "double_float") else "native"
        op = DslashOperator(dims, nd=4, prec=args.prec, recon=args.recon if kind == "dslash" else 18, spinor_format=fmt)
        if kind == "dslash" and args.variant >= 0:
            op.set_tuning(0, args.variant)
        u = su3_links(V * 4, gen, torch).to(dt).reshape(-1)
        psi = torch.randn(V * 24, dtype=dt, device="cuda", generator=gen)
    gauge = op.pack_gauge(u)
    src = op.pack_spinor(psi, 0)
    if kind == "force":
        chi = op.pack_spinor(psi, 1)
        f = torch.empty_like(u)
        launch = lambda: op.force(gauge, src, chi, 1, 0, f, mode=1)  # noqa: E731
    else:
        res = op.new_spinor()
        launch = lambda: op.apply(gauge, src, 1, 0, out=res)  # noqa: E731
    del u, psi
    for _ in range(args.warmup):
        launch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        launch()
    e1.record()
    torch.cuda.synchronize()
    op.check()
    print(json.dumps({"profile": kind, "dims": list(dims), "ms": e0.elapsed_time(e1) / args.steps,
                      "tuning": list(op.tuning()), "zblock": op.site_order()}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-solver", action="store_true")
    ap.add_argument("--variants", default="all",
                    help="comma list of variant sections: recon12, f64, 3d, multi_rhs, uneven_batch, force, split_t (default all)")
    ap.add_argument("--tuning", default=None,
                    help="block,variant of the headline kernel instead of autotuning (for profiling runs)")
    ap.add_argument("--dims", default=None,
                    help="Lx,Ly,Lz,Lt of the 4D workload (default 32,32,32,64; smaller cases are for profiling)")
    ap.add_argument("--profile", choices=["dslash", "force", "multi_rhs"], default=None,
                    help="build one operator on --dims and launch only its kernel (for ncu captures)")
    ap.add_argument("--prec", type=int, default=32, help="--profile dslash/force: 32 or 64")
    ap.add_argument("--recon", type=int, default=18, help="--profile dslash/multi_rhs: 18 or 12")
    ap.add_argument("--nrhs", type=int, default=32, help="--profile multi_rhs: right-hand sides")
    ap.add_argument("--fmt", default="bf16",
                    help="--profile multi_rhs: native, f32_pairs, bf16 or f16; --profile dslash --prec 64: double_float")
    ap.add_argument("--variant", type=int, default=-1, help="--profile: kernel variant (-1: the default)")
    ap.add_argument("--tc", action="store_true", help="--profile multi_rhs: the tensor-core kernel")
    ap.add_argument("--zblock", type=int, default=-1,
                    help="--profile multi_rhs: site order (z slab planes; 0 natural, -1 the default)")
    args = ap.parse_args()
    if args.dims:
        global DIMS, WORKLOAD
        DIMS = tuple(int(v) for v in args.dims.split(","))
        WORKLOAD = "wilson_dslash_4d_%dx%dx%dx%d_f32_recon18" % DIMS
    if args.warmup < 3:
        args.warmup = 3
    if args.profile:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
