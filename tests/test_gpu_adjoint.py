"""GPU adjoint: torch.autograd.Function gradients against the CPU adjoint of
the oracle and against central finite differences on 20 seeded directions
d ~ N(0, I).

Tolerance (1e-6 relative), stated per check:
  h = 1e-6: |g.d - FD| <= 1e-6 * max(|FD|, |g|_2).  |g|_2 is the standard
     deviation of g.d over the directions.  At this step the FD quotient of
     FP64 solves carries round-off of ~1e-12 relative to |g|_2 (error ~ 1/h),
     so a direction whose derivative is by chance 20x below typical cannot be
     resolved to 1e-6 of itself; measured on the oracle at 257^2: absolute FD
     error 1e-13..7e-13 for |g.d| from 6e-8 to 1.4e-6.
  h = 1e-5: |g.d - FD| <= 1e-6 * |FD| for every direction.
  h = 1e-6, per direction, with the difference of J written without
     cancellation, J(m+hd) - J(m-hd) = 0.5 sum (u+ - u-)(u+ + u- - 2 u_obs):
     median over the 20 directions <= 1e-6 * |FD|, every direction <= 2e-5 *
     |FD|.  The remaining floor is the round-off of the solutions themselves
     (about cond(A) * eps relative in u, against u+ - u- ~ h |du|): measured
     1.7e-7 median and 6.2e-6 worst, the same with the solves converged to
     1e-13 or to 1e-14.
"""
import numpy as np
import pytest

from helpers import oracle_params

pytestmark = pytest.mark.gpu


def _fd_check(J, grad, x0, ndir, h, seed, rtol, normwise):
    rng = np.random.default_rng(seed)
    worst = 0.0
    gnorm = float(np.linalg.norm(grad))
    for _ in range(ndir):
        d = rng.standard_normal(x0.shape[0])
        fd = (J(x0 + h * d) - J(x0 - h * d)) / (2 * h)
        ad = float(grad @ d)
        scale = max(abs(fd), gnorm) if normwise else abs(fd)
        worst = max(worst, abs(ad - fd) / max(scale, 1e-300))
    assert worst <= rtol, worst
    return worst


def _c3(ctx, nref, precision, rel_red):
    import torch
    from ugcore_gb300 import adjoint, problems
    cfg = problems.config("c3", nref=nref, precision=precision, rel_red=rel_red, maxit=500)
    prob = adjoint.DifferentiableProblem(ctx, cfg)
    m_true = torch.tensor(prob.m_top, device="cuda")
    f = torch.tensor(np.asarray([2.0 * _u(cfg["seed"], i) - 1.0 for i in range(prob.n)]), device="cuda")
    return cfg, prob, m_true, f


def _u(seed, i):
    from ugcore_gb300 import fields
    return fields.hash_uniform(seed, i)


def test_autograd_matches_oracle_adjoint(ctx, oracle_lib):
    import torch
    from ugcore_gb300 import adjoint
    cfg, prob, m_true, f = _c3(ctx, 4, "fp64", 1e-12)
    m = m_true * 0.7
    u = adjoint.fv1_solve(m.requires_grad_(), f, prob)
    uobs = torch.zeros_like(u)
    J = 0.5 * ((u - uobs) ** 2).sum()
    J.backward()
    gm = m.grad.cpu().numpy()
    op = oracle_lib.Problem(oracle_params(oracle_lib, dict(cfg, rel_red=1e-12)), m_top=m.detach().cpu().numpy(),
                            f_top=f.cpu().numpy())
    uo = op.solve()["x"]
    lam = op.adjoint(uo)["lam"]
    go = op.grad_logk(uo, lam)
    assert np.abs(u.detach().cpu().numpy() - uo).max() <= 1e-9 * np.abs(uo).max()
    assert np.abs(gm - go).max() <= 1e-8 * np.abs(go).max()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c3_gradient_vs_finite_differences(ctx, precision):
    """2D inverse problem, 257 x 257 vertices: J = 0.5 |u(m) - u_obs|^2 with
    u_obs = u(m_true) + 1% Gaussian noise."""
    import torch
    from ugcore_gb300 import adjoint
    cfg, prob, m_true, f = _c3(ctx, 7, precision, 1e-13)
    assert prob.n == 257 * 257
    with torch.no_grad():
        u_true = adjoint.fv1_solve(m_true, f, prob)
    rng = np.random.default_rng(7)
    noise = 0.01 * float(u_true.abs().max()) * torch.tensor(rng.standard_normal(prob.n), device="cuda")
    u_obs = u_true + noise
    m0 = (0.8 * m_true).clone().requires_grad_()
    u = adjoint.fv1_solve(m0, f, prob)
    J = 0.5 * ((u - u_obs) ** 2).sum()
    J.backward()
    g = m0.grad.cpu().numpy()

    def Jm(mm):
        with torch.no_grad():
            uu = adjoint.fv1_solve(torch.tensor(mm, device="cuda"), f, prob)
            return float(0.5 * ((uu - u_obs) ** 2).sum())

    x0 = m0.detach().cpu().numpy()
    _fd_check(Jm, g, x0, 20, 1e-6, 3, 1e-6, normwise=True)
    _fd_check(Jm, g, x0, 20, 1e-5, 4, 1e-6, normwise=False)

    # h = 1e-6 per direction, J's difference without cancellation
    def solve(mm):
        with torch.no_grad():
            return adjoint.fv1_solve(torch.tensor(mm, device="cuda"), f, prob).clone()
    rng = np.random.default_rng(3)
    h, rels = 1e-6, []
    for _ in range(20):
        d = rng.standard_normal(x0.shape[0])
        up, um = solve(x0 + h * d), solve(x0 - h * d)
        fd = float((0.5 * (up - um) * (up + um - 2 * u_obs)).sum()) / (2 * h)
        rels.append(abs(float(g @ d) - fd) / abs(fd))
    assert np.median(rels) <= 1e-6, rels
    assert max(rels) <= 2e-5, rels


def test_c4_source_gradient(ctx, oracle_lib):
    """convection-diffusion (full upwind, BiCGStab): dJ/df for J = sum of u^2
    over a seeded 10% vertex subset, against the oracle's adjoint and FD."""
    from ugcore_gb300 import problems
    cfg = problems.config("c4", nref=2, precision="fp64", rel_red=1e-13, maxit=400)
    p = problems.Problem(ctx, cfg)
    st = p.solve()
    assert st["converged"]
    u = p.x.numpy()
    rng = np.random.default_rng(cfg["seed"])
    S = rng.random(p.n) < 0.1
    g_u = np.where(S, 2.0 * u, 0.0)
    ast = p.adjoint_solve(g_u)
    assert ast["converged"]
    gf = p.disc.grad_source(p.lam)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg))
    uo = op.solve()["x"]
    lo = op.adjoint(np.where(S, 2.0 * uo, 0.0))["lam"]
    go = op.grad_source(lo)
    assert np.abs(gf - go).max() <= 1e-8 * np.abs(go).max()
    f0 = op.source()

    def Jf(ff):
        q = problems.Problem(ctx, cfg, f_top=ff)
        q.solve()
        return float(np.sum(q.x.numpy()[S] ** 2))

    _fd_check(Jf, gf, f0, 5, 1e-6, 5, 1e-6, normwise=True)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_repeated_gradients_reuse_the_adjoint_set_up(ctx, precision):
    """a gradient after an operator update re-initialises the kept transposed
    multigrid and solver: bit-identical to a fresh problem's gradient"""
    import torch
    from ugcore_gb300 import adjoint

    def grad(prob, m, f):
        mm = m.clone().requires_grad_(True)
        u = adjoint.fv1_solve(mm, f, prob)
        (0.5 * (u ** 2).sum()).backward()
        return mm.grad.cpu().numpy()

    cfg, prob, m_true, f = _c3(ctx, 4, precision, 1e-10)
    g1 = grad(prob, m_true * 0.7, f)
    g2 = grad(prob, m_true * 1.3, f)
    _, fresh, _, _ = _c3(ctx, 4, precision, 1e-10)
    g2_fresh = grad(fresh, m_true * 1.3, f)
    assert not np.array_equal(g1, g2)
    assert np.array_equal(g2.view(np.int64), g2_fresh.view(np.int64))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_recomputed_adjoint_equals_stored(ctx, precision):
    """adjoint_memory "recompute" (the forward operator and multigrid
    transposed in place for the adjoint, re-assembled for the next forward
    solve) gives the gradients of the stored transposed hierarchy to 1e-12,
    also after alternating forward and adjoint solves"""
    import torch
    from ugcore_gb300 import adjoint, problems

    def grads(mode):
        cfg = problems.config("c3", nref=5, precision=precision, adjoint_memory=mode)
        prob = adjoint.DifferentiableProblem(ctx, cfg)
        m0 = torch.tensor(prob.m_top, device="cuda")
        f = torch.ones(prob.n, dtype=torch.float64, device="cuda")
        out = []
        for s in (0.7, 1.3, 0.7):
            mm = (m0 * s).clone().requires_grad_(True)
            u = adjoint.fv1_solve(mm, f, prob)
            (0.5 * (u ** 2).sum()).backward()
            out.append(mm.grad.cpu().numpy())
        return out

    gs, gr = grads("store"), grads("recompute")
    for a, b in zip(gs, gr):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    assert np.array_equal(gr[0], gr[2])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_recomputed_adjoint_nonsymmetric(ctx, precision):
    """convection-diffusion (a non-symmetric operator): the adjoint solution
    of adjoint_memory "recompute" equals the stored variant's, in the same
    number of steps, before and after a forward solve in between"""
    from ugcore_gb300 import problems

    def lam(mode):
        p = problems.Problem(ctx, problems.config("c4", nref=3, precision=precision, adjoint_memory=mode))
        out = []
        for _ in range(2):
            p.solve()
            u = p.x.numpy()
            st = p.adjoint_solve(np.where(np.arange(p.n) % 7 == 0, u, 0.0))
            out.append((p.lam.numpy(), st["steps"]))
        return out

    for (a, sa), (b, sb) in zip(lam("store"), lam("recompute")):
        assert sa == sb
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_recomputed_adjoint_memory_c4_full_size(ctx):
    """193^3 convection-diffusion with the FP32 multigrid: the adjoint solve
    with adjoint_memory "recompute" holds no more than 1.15x the forward
    solve's device memory (the stored transposed hierarchy needs a second
    one), and its source gradient equals the stored variant's to 1e-12"""
    import torch
    from ugcore_gb300 import problems

    def run(mode):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        p = problems.Problem(ctx, problems.config("c4", adjoint_memory=mode))
        st = p.solve()
        assert st["converged"]
        ctx.synchronize()
        fwd = free0 - torch.cuda.mem_get_info()[0]
        u = p.x.numpy()
        S = np.random.default_rng(p.cfg["seed"]).random(p.n) < 0.1
        ast = p.adjoint_solve(np.where(S, 2.0 * u, 0.0))
        assert ast["converged"]
        g = p.disc.grad_source(p.lam)
        ctx.synchronize()
        both = free0 - torch.cuda.mem_get_info()[0]
        del p
        ctx.synchronize()
        return fwd, both, g

    f_r, b_r, g_r = run("recompute")
    f_s, b_s, g_s = run("store")
    print("c4 device memory: forward %.2f GB; with the adjoint: recompute %.2f GB, store %.2f GB"
          % (f_r / 1e9, b_r / 1e9, b_s / 1e9))
    assert b_r <= 1.15 * f_r, (b_r, f_r)
    assert b_s > 1.15 * f_s
    assert np.abs(g_r - g_s).max() <= 1e-12 * np.abs(g_s).max()
