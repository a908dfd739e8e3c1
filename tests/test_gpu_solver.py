"""Even-odd preconditioned operator and solvers (GPU), checked against the
oracle's Dslash: M x = x - kappa^2 D_eo D_oe x on the even sites."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

KAPPA = 0.124


def _even_M(dims, lol, u, x, kappa, isign):
    """Oracle: M (isign=+1) or M^+ (isign=-1) on the even sites, FP64."""
    t = O.dslash_plain(4, dims, lol, u, x, isign, 0)       # odd  <- even
    y = O.dslash_plain(4, dims, lol, u, t, isign, 1)       # even <- odd
    out = np.zeros_like(x)
    ev = O.target_sites(4, dims, lol, 1)
    out.reshape(-1, 24)[ev] = x.reshape(-1, 24)[ev] - kappa * kappa * y.reshape(-1, 24)[ev]
    return out, ev


@pytest.mark.parametrize("dagger", [False, True])
def test_apply_M_matches_oracle(dagger):
    import torch
    from sse_wilson_dslash_gb300.device import WilsonSolver
    dims = (8, 4, 6, 4)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, x = O.make_inputs(dims, 41, 42, kind="near_unit")
    s = WilsonSolver(dims, KAPPA, inner_prec=64)
    s.set_gauge(torch.from_numpy(u.ravel()).cuda())
    y = torch.full((x.size,), 7.0, dtype=torch.float64, device="cuda")
    s.apply(torch.from_numpy(x.ravel()).cuda(), y, dagger=dagger)
    ref, ev = _even_M(dims, lol, u, x, KAPPA, -1 if dagger else 1)
    got = y.cpu().numpy().reshape(-1, 24)
    odd = np.setdiff1d(np.arange(got.shape[0]), ev)
    assert np.all(got[odd] == 7.0)
    assert O.site_rel_err(got, ref, ev) < 1e-13
    s.close()


@pytest.mark.parametrize("inner_prec,inner_recon,outer_df", [(64, 18, False), (32, 18, False), (32, 12, False),
                                                              (32, 12, True), (16, 12, False), (16, 12, True),
                                                              (17, 12, False), (16, 18, False)])
def test_solve_reaches_tolerance(inner_prec, inner_recon, outer_df):
    """outer_df: the outer residual's operator in double-float instead of
    FP64; the oracle's FP64 residual checks both."""
    import torch
    from sse_wilson_dslash_gb300.device import WilsonSolver
    dims = (8, 8, 8, 8)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, b = O.make_inputs(dims, 51, 52, kind="near_unit")
    s = WilsonSolver(dims, KAPPA, tol=1e-10, inner_prec=inner_prec, inner_recon=inner_recon,
                     inner_tol=1e-5 if inner_prec >= 32 else 1e-3, outer_double_float=outer_df)
    s.set_gauge(torch.from_numpy(u.ravel()).cuda())
    x = torch.zeros(b.size, dtype=torch.float64, device="cuda")
    st = s.solve(torch.from_numpy(b.ravel()).cuda(), x)
    assert st["converged"] == 1 and st["residual"] <= 1e-10, st
    assert st["iterations"] > 5
    if inner_prec != 64:
        assert st["cycles"] >= 2
    # independent check: |b - M x| / |b| with the oracle's Dslash
    xv = x.cpu().numpy()
    Mx, ev = _even_M(dims, lol, u, xv, KAPPA, 1)
    bb = b.reshape(-1, 24)[ev]
    true_res = np.linalg.norm(bb - Mx.reshape(-1, 24)[ev]) / np.linalg.norm(bb)
    assert abs(true_res - st["true_residual"]) <= 1e-3 * true_res + 1e-14
    assert true_res < 1e-8
    s.close()


def test_mixed_and_fp64_solutions_agree():
    import torch
    from sse_wilson_dslash_gb300.device import WilsonSolver
    dims = (8, 8, 4, 8)
    u, b = O.make_inputs(dims, 61, 62, kind="near_unit")
    ut, bt = torch.from_numpy(u.ravel()).cuda(), torch.from_numpy(b.ravel()).cuda()
    xs = []
    for prec in (64, 32, 16, 17):
        s = WilsonSolver(dims, KAPPA, tol=1e-11, inner_prec=prec, inner_recon=12,
                         inner_tol=1e-5 if prec >= 32 else 1e-3)
        s.set_gauge(ut)
        x = torch.zeros_like(bt)
        assert s.solve(bt, x)["converged"] == 1
        xs.append(x)
        s.close()
    for x in xs[1:]:
        assert (xs[0] - x).norm() / xs[0].norm() < 1e-9


@pytest.mark.parametrize("nrhs,inner_recon,outer_df", [(4, 12, False), (8, 18, False), (16, 12, False),
                                                        (16, 12, True), (32, 18, False)])
def test_batched_solve_matches_single_solves(nrhs, inner_recon, outer_df):
    """The batched solver: every right-hand side reaches 1e-10, its solution
    agrees with the single-rhs mixed solve of the same system, and the
    oracle confirms |b - M x| / |b|.  One right-hand side is zero (its
    solution stays zero) and two are multiples of each other (their
    solutions are the same multiples).  16 and 32 right-hand sides run the
    fully packed operator with the CG's r update fused into M^+."""
    import torch
    from sse_wilson_dslash_gb300.device import BatchedWilsonSolver, WilsonSolver
    dims = (8, 8, 8, 8)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, _ = O.make_inputs(dims, 61, 62, kind="near_unit")
    rng = np.random.default_rng(63)
    bs = [O.gaussian_spinor(rng, V).ravel() for _ in range(nrhs)]
    bs[1] = np.zeros_like(bs[1])
    bs[3] = -2.5 * bs[2]
    bsolver = BatchedWilsonSolver(dims, nrhs, KAPPA, tol=1e-10, inner_recon=inner_recon, outer_double_float=outer_df)
    ug = torch.from_numpy(u.ravel()).cuda()
    bsolver.set_gauge(ug)
    bt = torch.from_numpy(np.stack(bs).ravel()).cuda()
    xt = torch.zeros_like(bt)
    stats = bsolver.solve(bt, xt)
    x = xt.cpu().numpy().reshape(nrhs, V * 24)
    single = WilsonSolver(dims, KAPPA, tol=1e-10, inner_prec=32, inner_recon=inner_recon, outer_double_float=outer_df)
    single.set_gauge(ug)
    ev = O.target_sites(4, dims, lol, 1)
    for q in range(nrhs):
        if q == 1:
            assert np.all(x[q] == 0.0) and stats[q]["iterations"] == 0
            continue
        assert stats[q]["converged"] == 1 and stats[q]["residual"] <= 1e-10, (q, stats[q])
        Mx, _ = _even_M(dims, lol, u, x[q], KAPPA, 1)
        num = np.linalg.norm((Mx - bs[q]).reshape(-1, 24)[ev])
        assert num / np.linalg.norm(bs[q].reshape(-1, 24)[ev]) < 1e-9, q
        xs = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
        single.solve(torch.from_numpy(bs[q].ravel()).cuda(), xs)
        xs = xs.cpu().numpy().reshape(-1, 24)[ev]
        assert np.linalg.norm(x[q].reshape(-1, 24)[ev] - xs) / np.linalg.norm(xs) < 1e-8, q
    np.testing.assert_allclose(x[3].reshape(-1, 24)[ev], -2.5 * x[2].reshape(-1, 24)[ev], rtol=0, atol=1e-8 * np.abs(x[3]).max())
    single.close()
    bsolver.close()


@pytest.mark.parametrize("scale", [1e30, 1e-30, 1.0])
def test_outer_residual_outside_the_double_float_range(scale):
    """With outer_double_float the outer residual b - M x runs in
    double-float (FP32 exponent range) when |b|^2 lies in [1e-50, 1e50] and
    on the FP64 operator otherwise:
    sources scaled by 1e30 and 1e-30 take the FP64 path, 1.0 the double-float
    one, and all three reach 1e-10 with the oracle's |b - M x| / |b| below
    1e-8; in the batched solver each rhs takes its own path (one scaled, one
    not)."""
    import torch
    from sse_wilson_dslash_gb300.device import BatchedWilsonSolver, WilsonSolver
    dims = (8, 8, 4, 8)
    V = O.volume(dims)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    u, b = O.make_inputs(dims, 71, 72, kind="near_unit")
    b = b.ravel() * scale
    ev = O.target_sites(4, dims, lol, 1)

    def true_res(xv, bv):
        Mx, _ = _even_M(dims, lol, u, xv, KAPPA, 1)
        return np.linalg.norm((Mx - bv.reshape(Mx.shape)).reshape(-1, 24)[ev]) / np.linalg.norm(bv.reshape(-1, 24)[ev])

    ug = torch.from_numpy(u.ravel()).cuda()
    s = WilsonSolver(dims, KAPPA, tol=1e-10, inner_prec=32, outer_double_float=True)
    s.set_gauge(ug)
    x = torch.zeros(b.size, dtype=torch.float64, device="cuda")
    st = s.solve(torch.from_numpy(b).cuda(), x)
    assert st["converged"] == 1 and st["residual"] <= 1e-10, st
    assert true_res(x.cpu().numpy(), b) < 1e-8
    s.close()
    rng = np.random.default_rng(73)
    b2 = np.stack([b, O.gaussian_spinor(rng, V).ravel()])
    bsolver = BatchedWilsonSolver(dims, 2, KAPPA, tol=1e-10, outer_double_float=True)
    bsolver.set_gauge(ug)
    xt = torch.zeros(b2.size, dtype=torch.float64, device="cuda")
    stats = bsolver.solve(torch.from_numpy(b2.ravel()).cuda(), xt)
    xb = xt.cpu().numpy().reshape(2, -1)
    for q in range(2):
        assert stats[q]["converged"] == 1, (q, stats[q])
        assert true_res(xb[q], b2[q]) < 1e-8, q
    bsolver.close()


@pytest.mark.slow
def test_batched_solve_in_z_slabs_matches_single_solves():
    """24^3x48 with 32 rhs: the batched solver's operator runs in z slabs of
    12 planes (its FP32-pair fields' reuse span exceeds the L2 budget), the
    fused xpay and CG-update epilogues included; rhs 0 and 31 agree with
    single-rhs solves (natural site order) to 1e-8 and reach 1e-10."""
    import torch
    from bench import near_unit_links
    from sse_wilson_dslash_gb300.device import BatchedWilsonSolver, DslashOperator, WilsonSolver
    dims = (24, 24, 24, 48)
    V = O.volume(dims)
    probe = DslashOperator(dims, nd=4, prec=32, recon=12, nrhs=32, spinor_format="f32_pairs")
    assert probe.site_order() == 12
    probe.close()
    gen = torch.Generator(device="cuda").manual_seed(81)
    u = near_unit_links(V * 4, gen, torch).reshape(-1)
    b = torch.randn(32, V * 24, dtype=torch.float64, device="cuda", generator=gen)
    bs = BatchedWilsonSolver(dims, 32, KAPPA, tol=1e-10, inner_recon=12)
    bs.set_gauge(u)
    x = torch.zeros_like(b)
    stats = bs.solve(b, x)
    bs.close()
    assert all(t["converged"] == 1 for t in stats)
    single = WilsonSolver(dims, KAPPA, tol=1e-10, inner_prec=32, inner_recon=12)
    single.set_gauge(u)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    ev = torch.from_numpy(O.target_sites(4, dims, lol, 1)).cuda()
    for q in (0, 31):
        xs = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
        st = single.solve(b[q], xs)
        assert st["converged"] == 1
        a, c = x[q].view(V, 24)[ev], xs.view(V, 24)[ev]
        assert ((a - c).norm() / c.norm()).item() < 1e-8, q
    single.close()


def test_batched_solver_rejects_bad_arguments():
    from sse_wilson_dslash_gb300 import _lib
    from sse_wilson_dslash_gb300.device import BatchedWilsonSolver
    for kw in ({"nrhs": 3}, {"nrhs": 64}):
        with pytest.raises(_lib.GbdsError):
            BatchedWilsonSolver((4, 4, 4, 4), kw["nrhs"], KAPPA)
