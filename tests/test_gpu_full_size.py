"""Every benchmark configuration at its stated size against the oracle.

  c0  2D Poisson, 2x2 quads refined 6x (129^2 = 16,641 DoFs), FP64
  c1  3D Poisson, 2x2x2 hexes refined 6x (129^3 = 2,146,689 DoFs), FP64 and
      the FP32 multigrid
  c2  3D lognormal K on 4^3 hexes x 6 Kuhn tets refined 5x (129^3 vertices),
      FP64 and the FP32 multigrid
  c3  2D inverse problem, 257^2 quads: forward solve and the adjoint gradient
      dJ/dm through torch.autograd against the oracle's adjoint
  c4  3D convection-diffusion, 3^3 hexes refined 6x (193^3 = 7,189,057
      DoFs), BiCGStab, FP64 and the FP32 multigrid, and the adjoint dJ/df

Bars (the parity contract of this path): CRS row pointers and columns
bit-exact, values 1e-13 relative to the row's largest entry, transfers P/R
bit-exact, FP64 multigrid application 1e-12, FP64 solves within +-1
iterations of the oracle with the defect history to 1e-6 relative (down to
1e-6 of the initial defect; within a factor 2 below, where rounding
differences of the summation order dominate) and the solution to 1e-8; the FP32 multigrid within +-1 iterations of the GPU FP64
path, relative residual < 1e-10 in FP64 and its error against the FP64
oracle solution below 1e-7 (printed per configuration); adjoint gradients
1e-8 relative to the oracle's in FP64.

The oracle runs single-threaded: c1 takes about 10 s, c4 a minute or two.
Its results are computed once per module and shared by the FP64 and FP32
checks of a configuration.
"""
import numpy as np
import pytest

from helpers import assert_crs_equal, oracle_params, rel_residual

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def cache():
    return {}


def _oracle(orc, cache, name, cfg, m_top=None):
    """(oracle problem, its FP64 solve) of a configuration, computed once"""
    if name not in cache:
        op = orc.Problem(oracle_params(orc, cfg), m_top=m_top)
        cache[name] = (op, op.solve(hist_cap=1000))
    return cache[name]


def _check_history(h, ref):
    """defect histories: 1e-6 relative while the defect is above 1e-6 of the
    initial one; below that the two FP64 iterations (GPU reductions sum in
    another order than the sequential oracle, the operators agree to
    rounding) drift apart, amplified by the conditioning (the
    lognormal-coefficient problem: 2e-6 at 2e-7 of the initial defect, ~10% at
    1e-10 after 40 steps), so only a factor of 2 is required there"""
    early = ref >= 1e-6 * ref[0]
    assert np.allclose(h[early], ref[early], rtol=1e-6, atol=0)
    ratio = h[~early] / ref[~early]
    assert np.all((ratio > 0.5) & (ratio < 2.0)), ratio


def _fp64_vs_oracle(ctx, orc, cache, name, check_levels=True):
    from ugcore_gb300 import problems
    cfg = problems.config(name, precision="fp64")
    p = problems.Problem(ctx, cfg)
    op, ref = _oracle(orc, cache, name, cfg, m_top=getattr(p, "m_top", None))
    assert p.n == op.nv()
    assert_crs_equal(p.A.export_csr(), op.matrix(), what="%s top operator" % name)
    b, ob = p.b.numpy(), op.rhs()
    assert np.abs(b - ob).max() <= 1e-13 * np.abs(ob).max()
    if check_levels:
        for l in range(1, p.hier.num_levels):
            for which in (0, 1):
                assert_crs_equal(p.gmg.transfer(l, which), op.transfer(l, which), rtol=0.0,
                                 what="%s %s level %d" % (name, "PR"[which], l))
    st = p.solve()
    assert st["converged"] and ref["converged"]
    assert abs(st["steps"] - ref["steps"]) <= 1, (st["steps"], ref["steps"])
    x = p.x.numpy()
    assert rel_residual(p, x) < 1e-10
    err = np.abs(x - ref["x"]).max() / np.abs(ref["x"]).max()
    assert err <= 1e-8, err
    h = p.solver.history()
    n = min(len(h), len(ref["history"]))
    _check_history(h[:n], ref["history"][:n])
    print("%s FP64 full size: %d DoFs, %d steps (oracle %d), |x - x_oracle|/|x| = %.2e"
          % (name, p.n, st["steps"], ref["steps"], err))
    return p, st


def _mixed_vs_fp64(ctx, orc, cache, name, steps64):
    from ugcore_gb300 import problems
    cfg = problems.config(name, precision="mixed")
    p = problems.Problem(ctx, cfg)
    _, ref = _oracle(orc, cache, name, problems.config(name, precision="fp64"), m_top=getattr(p, "m_top", None))
    st = p.solve()
    x = p.x.numpy()
    assert st["converged"] and rel_residual(p, x) < 1e-10
    assert abs(st["steps"] - steps64) <= 1, (st["steps"], steps64)
    err = np.abs(x - ref["x"]).max() / np.abs(ref["x"]).max()
    print("%s mixed full size: %d steps (GPU FP64 %d, oracle FP64 %d), max rel error vs FP64 oracle %.2e"
          % (name, st["steps"], steps64, ref["steps"], err))
    assert err < 1e-7, err
    return p


def test_c0_full_size(ctx, oracle_lib, cache):
    import ugcore_gb300 as ug
    p, _ = _fp64_vs_oracle(ctx, oracle_lib, cache, "c0")
    assert p.n == 129 * 129
    op, _ = cache["c0"]
    d = np.random.default_rng(10).standard_normal(p.n)
    d[p.hier.export()[2].astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def test_c1_full_size_fp64_and_mixed(ctx, oracle_lib, cache):
    import ugcore_gb300 as ug
    p, st = _fp64_vs_oracle(ctx, oracle_lib, cache, "c1")
    assert p.n == 129 ** 3
    op, _ = cache["c1"]
    d = np.random.default_rng(11).standard_normal(p.n)
    d[p.hier.export()[2].astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    del p
    _mixed_vs_fp64(ctx, oracle_lib, cache, "c1", st["steps"])


def test_c2_full_size_fp64_and_mixed(ctx, oracle_lib, cache):
    p, st = _fp64_vs_oracle(ctx, oracle_lib, cache, "c2")
    assert p.n == 129 ** 3
    del p
    _mixed_vs_fp64(ctx, oracle_lib, cache, "c2", st["steps"])


def test_c4_full_size_fp64_mixed_and_adjoint(ctx, oracle_lib, cache):
    """193^3 convection-diffusion: FP64 BiCGStab against the oracle's
    (iterations +-1, solution, history), the FP32 multigrid against it, and
    the adjoint dJ/df of J = sum of u^2 over a seeded 10% vertex subset
    (transposed BiCGStab + source gradient) against the oracle's adjoint"""
    from ugcore_gb300 import problems
    p, st = _fp64_vs_oracle(ctx, oracle_lib, cache, "c4", check_levels=False)
    assert p.n == 193 ** 3
    op, ref = cache["c4"]
    S = np.random.default_rng(p.cfg["seed"]).random(p.n) < 0.1
    ast = p.adjoint_solve(np.where(S, 2.0 * p.x.numpy(), 0.0))
    assert ast["converged"]
    gf = p.disc.grad_source(p.lam)
    ra = op.adjoint(np.where(S, 2.0 * ref["x"], 0.0))
    assert ra["converged"]
    assert abs(ast["steps"] - ra["steps"]) <= 1, (ast["steps"], ra["steps"])
    go = op.grad_source(ra["lam"])
    gerr = np.abs(gf - go).max() / np.abs(go).max()
    print("c4 adjoint full size: %d half steps (oracle %d), |g - g_oracle|/|g| = %.2e"
          % (ast["steps"], ra["steps"], gerr))
    assert gerr <= 1e-8, gerr
    del p
    pm = _mixed_vs_fp64(ctx, oracle_lib, cache, "c4", st["steps"])
    um = pm.x.numpy()
    am = pm.adjoint_solve(np.where(S, 2.0 * um, 0.0))
    assert am["converged"]
    gm = pm.disc.grad_source(pm.lam)
    merr = np.abs(gm - go).max() / np.abs(go).max()
    print("c4 mixed adjoint: max rel error of dJ/df vs the FP64 oracle %.2e" % merr)
    assert merr < 1e-6, merr
    assert problems.config("c4")["precision"] == "mixed"


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-6)])
def test_c3_full_size_forward_and_adjoint(ctx, oracle_lib, cache, precision, tol):
    """257^2 inverse problem at m = m_true (the seeded 32-mode field), source
    f ~ U[-1,1]: the forward solve against the oracle's, and the gradient
    of J = 0.5 |u - u_obs|^2 (u_obs = the oracle solution plus 1% noise)
    through torch.autograd against the oracle's adjoint gradient"""
    import torch
    from ugcore_gb300 import adjoint, fields, problems
    cfg = problems.config("c3", precision=precision)
    prob = adjoint.DifferentiableProblem(ctx, cfg)
    assert prob.n == 257 * 257
    f = np.asarray([2.0 * fields.hash_uniform(cfg["seed"], i) - 1.0 for i in range(prob.n)])
    op = oracle_lib.Problem(oracle_params(oracle_lib, dict(cfg, precision="fp64")), m_top=prob.m_top, f_top=f)
    ref = op.solve()
    assert ref["converged"]
    noise = 0.01 * np.abs(ref["x"]).max() * np.random.default_rng(3).standard_normal(prob.n)
    u_obs_np = ref["x"] + noise
    m = torch.tensor(prob.m_top, device="cuda", requires_grad=True)
    ft = torch.tensor(f, device="cuda")
    u = adjoint.fv1_solve(m, ft, prob)
    st = prob.solver.stats()
    uerr = np.abs(u.detach().cpu().numpy() - ref["x"]).max() / np.abs(ref["x"]).max()
    if precision == "fp64":
        assert abs(st["steps"] - ref["steps"]) <= 1, (st["steps"], ref["steps"])
    assert uerr <= tol, uerr
    u_obs = torch.tensor(u_obs_np, device="cuda")
    (0.5 * ((u - u_obs) ** 2).sum()).backward()
    g = m.grad.cpu().numpy()
    lam = op.adjoint(ref["x"] - u_obs_np)
    assert lam["converged"]
    go = op.grad_logk(ref["x"], lam["lam"])
    gerr = np.abs(g - go).max() / np.abs(go).max()
    print("c3 %s full size: %d CG steps (oracle %d), |u - u_oracle|/|u| = %.2e, |g - g_oracle|/|g| = %.2e"
          % (precision, st["steps"], ref["steps"], uerr, gerr))
    assert gerr <= tol, gerr
