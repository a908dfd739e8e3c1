"""Adjoint and force (GPU): dL/dpsi and dL/dU of L = Re <chi, D psi> and of
S = phi^+ (M^+M)^-1 phi, against an FP64 numpy gradient, FP64 central finite
differences (step 1e-6) along random su(3) directions, and torch.autograd.gradcheck."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS = 1e-6


def _rand_su3_algebra(rng, n):
    a = rng.standard_normal((n, 3, 3)) + 1j * rng.standard_normal((n, 3, 3))
    X = (a - np.conj(np.swapaxes(a, -1, -2))) / 2
    tr = np.trace(X, axis1=-2, axis2=-1) / 3
    X -= tr[:, None, None] * np.eye(3)
    return X


def _expm_antiherm(X, eps):
    H = -1j * X                      # Hermitian
    w, v = np.linalg.eigh(H)
    return np.einsum("nij,nj,nkj->nik", v, np.exp(1j * eps * w), np.conj(v))


def _perturb(u, X, eps):
    """packed u -> packed exp(eps X) U (X per link, [V*4,3,3])."""
    U = O.unpack_links(u).reshape(-1, 3, 3)
    Up = np.einsum("nij,njk->nik", _expm_antiherm(X, eps), U)
    return O.pack_links(Up.reshape(u.shape[0], 4, 3, 3))


def _gpu(op, u):
    import torch
    return op.pack_gauge(torch.from_numpy(np.ascontiguousarray(u).ravel()).cuda())


def _L(op, u, psi, chi, isign, cb):
    """Re <chi, D psi> on the target sites, FP64 on the GPU."""
    import torch
    gauge = _gpu(op, u)
    out = op.apply(gauge, op.pack_spinor(torch.from_numpy(psi.ravel()).cuda(), cb), isign, cb)
    res = torch.zeros(psi.size, dtype=torch.float64, device="cuda")
    op.unpack_spinor(out, 1 - cb, res)
    return float(torch.dot(res, torch.from_numpy(chi.ravel()).cuda()))


def _numpy_gradient(dims, u, psi, chi, isign, cb):
    """Complex gradient G[V,4,i,j] of Re <chi, D psi> (lexicographic -> cb2 order)."""
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    U, P = O.to_lex_fields(dims, lol, u, psi)
    _, C = O.to_lex_fields(dims, lol, u, chi)
    g = O.gamma_matrices()
    par = O.parity_of_lex(dims, 4).reshape(P.shape[:4])
    tgt, src = par == 1 - cb, par == cb
    axis = {0: 3, 1: 2, 2: 1, 3: 0}
    G = np.zeros(U.shape, dtype=np.complex128)
    for mu in range(4):
        pm, pp = np.eye(4) - isign * g[mu], np.eye(4) + isign * g[mu]
        phi = np.einsum("st,...tj->...sj", pm, np.roll(P, -1, axis=axis[mu]))
        Gf = np.einsum("...si,...sj->...ij", C, np.conj(phi))
        phib = np.einsum("st,...tj->...sj", pp, P)
        Gb = np.einsum("...si,...sj->...ij", phib, np.conj(np.roll(C, -1, axis=axis[mu])))
        G[mu] = np.where(tgt[..., None, None], Gf, 0) + np.where(src[..., None, None], Gb, 0)
    out = np.zeros((O.volume(dims), 4, 3, 3), dtype=np.complex128)
    out[lol] = np.moveaxis(G, 0, 4).reshape(-1, 4, 3, 3)
    return out


def _unpack_complex(f):
    return O.unpack_links(f.reshape(-1, 4, 3, 3, 2))  # [V,4,i,j]


@pytest.mark.parametrize("dims", [(4, 4, 2, 4), (16, 16, 16, 16)])
@pytest.mark.parametrize("isign,cb", [(1, 0), (-1, 1)])
def test_gradient_matches_numpy(isign, cb, dims):
    """The complex gradient dL/dU of every link (mode 0) against the FP64
    numpy gradient; 16^4 is the configured FP64 size."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    rng = np.random.default_rng(5)
    V = O.volume(dims)
    u = O.random_gauge(rng, V)
    psi, chi = O.gaussian_spinor(rng, V), O.gaussian_spinor(rng, V)
    op = DslashOperator(dims, prec=64)
    gauge = _gpu(op, u)
    ps = op.pack_spinor(torch.from_numpy(psi.ravel()).cuda(), cb)
    cs = op.pack_spinor(torch.from_numpy(chi.ravel()).cuda(), 1 - cb)
    out = torch.zeros(V * 72, dtype=torch.float64, device="cuda")
    op.force(gauge, ps, cs, isign, cb, out, mode=0)
    G = _unpack_complex(out.cpu().numpy())
    ref = _numpy_gradient(dims, u, psi, chi, isign, cb)
    assert np.max(np.abs(G - ref)) < 1e-12 * np.max(np.abs(ref))
    op.close()


def _force(dims, prec, u, psi, chi, isign, cb):
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    V = O.volume(dims)
    op = DslashOperator(dims, prec=prec)
    dt = torch.float64 if prec == 64 else torch.float32
    gauge = op.pack_gauge(torch.from_numpy(u.ravel()).to(dt).cuda())
    ps = op.pack_spinor(torch.from_numpy(psi.ravel()).to(dt).cuda(), cb)
    cs = op.pack_spinor(torch.from_numpy(chi.ravel()).to(dt).cuda(), 1 - cb)
    out = torch.zeros(V * 72, dtype=dt, device="cuda")
    op.force(gauge, ps, cs, isign, cb, out, mode=1)
    return _unpack_complex(out.double().cpu().numpy()).reshape(-1, 3, 3)


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (16, 16, 16, 16)])
@pytest.mark.parametrize("isign,cb", [(1, 0), (-1, 1)])
def test_force_matches_finite_differences(isign, cb, dims):
    """The su(3) force (mode 1) against FP64 central differences of L along a
    random su(3) direction on every link (step 1e-6); 16^4 is the configured
    FP64 size."""
    from sse_wilson_dslash_gb300.device import DslashOperator
    rng = np.random.default_rng(6)
    V = O.volume(dims)
    u = O.random_gauge(rng, V)
    psi, chi = O.gaussian_spinor(rng, V), O.gaussian_spinor(rng, V)
    X = _rand_su3_algebra(rng, V * 4)
    op64 = DslashOperator(dims, prec=64)
    fd = (_L(op64, _perturb(u, X, EPS), psi, chi, isign, cb) -
          _L(op64, _perturb(u, X, -EPS), psi, chi, isign, cb)) / (2 * EPS)
    F = _force(dims, 64, u, psi, chi, isign, cb)
    # traceless anti-Hermitian
    assert np.max(np.abs(F + np.conj(np.swapaxes(F, -1, -2)))) < 1e-12
    assert np.max(np.abs(np.trace(F, axis1=-2, axis2=-1))) < 1e-12
    pred = float(np.sum(np.real(np.conj(F) * X)))  # Re tr(F^+ X)
    assert abs(pred - fd) <= 1e-7 * abs(fd), (pred, fd)
    # the FP32 force agrees with the FP64 one to FP32 rounding
    F32 = _force(dims, 32, u, psi, chi, isign, cb)
    assert np.max(np.abs(F32 - F)) <= 2e-6 * np.max(np.abs(F))


def test_dL_dpsi_is_dslash_dagger():
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (4, 4, 4, 4)
    rng = np.random.default_rng(8)
    V = O.volume(dims)
    u = O.random_gauge(rng, V)
    psi, chi, d = (O.gaussian_spinor(rng, V) for _ in range(3))
    op = DslashOperator(dims, prec=64)
    fd = (_L(op, u, psi + EPS * d, chi, 1, 0) - _L(op, u, psi - EPS * d, chi, 1, 0)) / (2 * EPS)
    gauge = _gpu(op, u)
    g = op.apply(gauge, op.pack_spinor(torch.from_numpy(chi.ravel()).cuda(), 1), -1, 1)
    grad = torch.zeros(V * 24, dtype=torch.float64, device="cuda")
    op.unpack_spinor(g, 0, grad)
    pred = float(np.dot(grad.cpu().numpy(), d.ravel()))
    assert abs(pred - fd) <= 1e-8 * abs(fd)


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (16, 16, 16, 16)])
def test_solver_force_matches_finite_differences(dims):
    """S = phi^+ (M^+M)^-1 phi, M = 1 - kappa^2 D_eo D_oe:
    dS = 2 kappa^2 (Re<Y, dD_eo Z> + Re<W, dD_oe X>), X = (M^+M)^-1 phi,
    Y = M X, Z = D_oe X, W = D_eo^+ Y.  16^4 is the configured FP64 size."""
    import torch
    from sse_wilson_dslash_gb300.device import DslashOperator, WilsonSolver
    kappa = 0.124
    rng = np.random.default_rng(9)
    V = O.volume(dims)
    u = O.random_gauge(rng, V, kind="near_unit")
    phi = O.gaussian_spinor(rng, V)
    lol = O.layout_table(O.LAYOUT_CB2, dims)
    ev = O.target_sites(4, dims, lol, 1)
    phi.reshape(V, 24)[np.setdiff1d(np.arange(V), ev)] = 0.0
    phit = torch.from_numpy(phi.ravel()).cuda()

    def S(uu):
        s = WilsonSolver(dims, kappa, tol=1e-12, max_iter=5000, inner_prec=64)
        s.set_gauge(torch.from_numpy(np.ascontiguousarray(uu).ravel()).cuda())
        x = torch.zeros_like(phit)
        st = s.solve(phit, x, normal=True)
        assert st["residual"] <= 1e-11, st
        s.close()
        return float(torch.dot(phit, x)), x

    Xdir = _rand_su3_algebra(rng, V * 4)
    fd = (S(_perturb(u, Xdir, EPS))[0] - S(_perturb(u, Xdir, -EPS))[0]) / (2 * EPS)
    _, Xsol = S(u)
    op = DslashOperator(dims, prec=64)
    gauge = _gpu(op, u)
    Xi = op.pack_spinor(Xsol, 0)
    Z = op.apply(gauge, Xi, 1, 0)                      # odd
    Y = op.new_spinor()
    # Y = X - kappa^2 D_eo Z
    DZ = op.apply(gauge, Z, 1, 1)
    Yp = torch.zeros_like(phit)
    Xp = torch.zeros_like(phit)
    op.unpack_spinor(DZ, 0, Yp)
    op.unpack_spinor(Xi, 0, Xp)
    Yp = Xp - kappa * kappa * Yp
    Y = op.pack_spinor(Yp, 0)
    W = op.apply(gauge, Y, -1, 0)                      # odd: D_eo^+ Y
    force = torch.zeros(V * 72, dtype=torch.float64, device="cuda")
    op.force(gauge, Z, Y, 1, 1, force, mode=1, coef=2 * kappa * kappa)
    op.force(gauge, Xi, W, 1, 0, force, mode=1, coef=2 * kappa * kappa, accumulate=True)
    F = _unpack_complex(force.cpu().numpy()).reshape(-1, 3, 3)
    pred = float(np.sum(np.real(np.conj(F) * Xdir)))
    assert abs(pred - fd) <= 1e-5 * abs(fd), (pred, fd)


def test_autograd_gradcheck():
    import torch
    from autograd_dslash import DslashFn
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (2, 2, 2, 2)
    V = O.volume(dims)
    op = DslashOperator(dims, prec=64)
    g = torch.Generator(device="cuda").manual_seed(1)
    u = torch.randn(V * 72, dtype=torch.float64, device="cuda", generator=g, requires_grad=True)
    psi = torch.randn(V * 24, dtype=torch.float64, device="cuda", generator=g, requires_grad=True)
    for isign, cb in ((1, 0), (-1, 1)):
        assert torch.autograd.gradcheck(lambda a, b: DslashFn.apply(a, b, op, isign, cb), (u, psi),
                                        eps=1e-6, atol=1e-8, rtol=1e-6)


@pytest.mark.slow
@pytest.mark.parametrize("isign,cb", [(1, 0), (-1, 1)])
def test_fp32_force_32x32x32x64_matches_fp64(isign, cb):
    """At the configured FP32 size, 32^3x64, the FP32 su(3) force of every link
    against the FP64 force of the same inputs: the largest per-link
    difference is at most 2e-6 of the largest per-link force, and the
    difference over all links at most 1e-6 of the force (Frobenius norms;
    FP32 rounding of the inputs and of the arithmetic, unit 6e-8)."""
    import torch
    from bench import su3_links
    from sse_wilson_dslash_gb300.device import DslashOperator
    dims = (32, 32, 32, 64)
    V = O.volume(dims)
    gen = torch.Generator(device="cuda").manual_seed(12)
    u = su3_links(V * 4, gen, torch).reshape(-1)
    psi = torch.randn(V * 24, dtype=torch.float64, device="cuda", generator=gen)
    chi = torch.randn(V * 24, dtype=torch.float64, device="cuda", generator=gen)
    forces = {}
    for prec, dt in ((64, torch.float64), (32, torch.float32)):
        op = DslashOperator(dims, prec=prec)
        gauge = op.pack_gauge(u.to(dt))
        ps = op.pack_spinor(psi.to(dt), cb)
        cs = op.pack_spinor(chi.to(dt), 1 - cb)
        out = torch.zeros(V * 72, dtype=dt, device="cuda")
        op.force(gauge, ps, cs, isign, cb, out, mode=1)
        torch.cuda.synchronize()
        forces[prec] = out.double().view(V * 4, 18)
        del gauge, ps, cs
        op.close()
    d = (forces[32] - forces[64]).norm(dim=1)
    f = forces[64].norm(dim=1)
    assert d.max().item() <= 2e-6 * f.max().item(), (d.max().item(), f.max().item())
    assert d.norm().item() <= 1e-6 * f.norm().item()
