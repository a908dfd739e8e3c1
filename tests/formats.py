"""Stored values and per-site error bounds of the spinor storage formats,
shared by the multi-RHS and batch tests.

Per-site bounds ||got - ref|| / ||ref||, where ref is the oracle applied to the
inputs as the field stores them (``stored``):

* FP32 (native, spin pairs): the parity tests' 1e-6;
* CUDA-core kernels with 16-bit storage round only the output:
  - bfloat16 rounds each component to nearest with 8 significant bits, an
    error of at most 2^-8 = 3.9e-3 of the component and so of the site's
    norm; with FP32 arithmetic, 4e-3;
  - half + norm stores v * (1/m) in half (11 significant bits, at most 2^-11
    of each component; values below half's normal range lose at most 2^-25 m),
    m the site's largest component: about 5e-4 of the site's norm; 1e-3;
* the tensor-core kernel also rounds the projected half spinors and the links
  to the 16-bit operand type before its FP32-accumulating MMAs: 1.2e-2
  (bfloat16) and 3e-3 (half).
"""
import numpy as np

TOL = {"native": 1e-6, "f32_pairs": 1e-6, "bf16": 4e-3, "f16": 1e-3}
TOL_TC = {"bf16": 1.2e-2, "f16": 3e-3}


def stored(psi, fmt):
    """FP64 values that a field of format ``fmt`` holds for the FP32 spinors
    ``psi`` (last axes [V][4][3][2] or [V][24]), rounded the way the pack
    kernels round them: bfloat16 to nearest; half + norm as
    half(v * (1 / m)) * m with m the site's largest |component|."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(psi, dtype=np.float32))
    if fmt == "bf16":
        return t.to(torch.bfloat16).double().numpy()
    if fmt == "f16":
        v = t.reshape(-1, 24)
        m = v.abs().amax(1, keepdim=True)
        inv = torch.where(m > 0, 1.0 / torch.where(m > 0, m, torch.ones_like(m)), torch.zeros_like(m))
        q = (v * inv).half().float() * m
        return q.reshape(t.shape).double().numpy()
    return t.double().numpy()


def site_err(got, ref, sites):
    """max over right-hand sides and ``sites`` of the per-site relative error
    (got, ref: [nrhs][V][24])."""
    g = np.asarray(got, dtype=np.float64)[:, sites]
    r = np.asarray(ref, dtype=np.float64)[:, sites]
    num = np.sqrt(((g - r) ** 2).sum(-1))
    den = np.sqrt((r ** 2).sum(-1))
    return float((num / np.maximum(den, 1e-300)).max())
