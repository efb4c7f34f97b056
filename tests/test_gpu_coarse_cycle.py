"""The coarse end of a V-cycle in one launch (k_coarse.cu) against separate
launches per smoothing step, transfer and base solve.

Every row of the one-block cycle uses the arithmetic of the separate kernels,
so multigrid corrections must be bit-identical, and the Krylov solves that
use them must take the same steps with the same defect history and the same
solution bits.  Cases cover 9-, 15- and 27-diagonal operators (quads, Kuhn
tets, hexes), upwind convection, ragged level sizes, every smoothing count
from 0 to 3 on either side, damped transfers, FP64 and FP32 levels, Galerkin coarse operators
and the transposed multigrid of the adjoint.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("c3", dict(nref=5), "fp64"),
    ("c3", dict(nref=5), "mixed"),
    ("c3", dict(nref=4, mx=3, my=5), "fp64"),                        # ragged 49 x 81
    ("c3", dict(nref=5, nu1=1, nu2=3), "fp64"),
    ("c3", dict(nref=5, nu1=0, nu2=2), "mixed"),
    ("c3", dict(nref=5, nu1=3, nu2=0), "fp64"),
    ("c3", dict(nref=5, damp_prol=0.8, damp_res=0.9), "mixed"),
    ("c3", dict(nref=5, base=1), "fp64"),                            # 5 x 5 base level
    ("c0", dict(nref=5, mx=5, my=2), "fp64"),                        # ragged 161 x 65
    ("c1", dict(nref=3), "fp64"),                                     # 27 diagonals
    ("c1", dict(nref=3), "mixed"),
    ("c2", dict(nref=3), "mixed"),                                    # 15 diagonals
    ("c2", dict(nref=2, mx=3, my=5, mz=2), "fp64"),                  # ragged 13 x 21 x 9
    ("c4", dict(nref=3), "mixed"),                                    # upwind convection
    ("c3", dict(nref=5, rap=True), "fp64"),                           # Galerkin coarse operators
    ("c2", dict(nref=3, rap=True), "mixed"),
]


def _problem(levels, name, over, prec):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    ctx = ug.Context(0)
    ctx.set_tuning(coarse_levels=levels)
    return problems.Problem(ctx, problems.config(name, precision=prec, **over))


def _coarse_launches(p, fn):
    p.ctx.profile_begin()
    fn()
    prof = p.ctx.profile_end()
    return sum(v[0] for k, v in prof.items() if "k_coarse_cycle" in k)


def _apply(p, d):
    import ugcore_gb300 as ug
    dv = ug.GPUVector(p.ctx, p.n).copy_from(d)
    cv = ug.GPUVector(p.ctx, p.n)
    p.gmg.apply(cv, dv)
    return cv, dv


@pytest.mark.parametrize("name,over,prec", CASES)
def test_gmg_application_bit_identical(name, over, prec):
    ref = _problem(0, name, over, prec)
    d = np.random.default_rng(11).uniform(-1.0, 1.0, ref.n)
    cr, dr = _apply(ref, d)
    want = cr.numpy()
    assert _coarse_launches(ref, lambda: ref.gmg.apply(cr, dr)) == 0
    fused_any = False
    for levels in (-1, 1, 2, 3, 7):
        p = _problem(levels, name, over, prec)
        cv, dv = _apply(p, d)
        got = cv.numpy()
        assert np.array_equal(got, want), (levels, float(np.abs(got - want).max()))
        nl = _coarse_launches(p, lambda: p.gmg.apply(cv, dv))
        assert nl in (0, 1)
        if levels > 0 and not over.get("rap"):
            assert nl == 1, levels   # every case has at least one level between base and top
        fused_any |= nl == 1
        # a second application (graph replay) gives the same bits
        p.gmg.apply(cv, dv)
        assert np.array_equal(cv.numpy(), want)
    # Galerkin levels are fused only where their stencil width is one the
    # kernel is built for (9, 15, 27) and the same on every fused level
    assert fused_any or over.get("rap")


@pytest.mark.parametrize("name,over,prec", [CASES[0], CASES[1], CASES[9], CASES[11], CASES[13]])
def test_solve_identical(name, over, prec):
    ref = _problem(0, name, over, prec)
    p = _problem(-1, name, over, prec)
    s1, s2 = ref.solve(), p.solve()
    assert s1["steps"] == s2["steps"]
    assert s1["defect"] == s2["defect"]
    assert np.array_equal(ref.solver.history(), p.solver.history())
    assert np.array_equal(ref.x.numpy(), p.x.numpy())


def test_not_used_outside_its_domain():
    """W and F cycles, Gauss-Seidel smoothers and a smoothing base solver keep
    the separate launches (and their results)"""
    for over in (dict(cycle=2), dict(cycle=-1), dict(smoother="mcsgs"), dict(base_solver="smoother", base_steps=3)):
        p = _problem(7, "c3", dict(nref=4, **over), "fp64")
        cv, dv = _apply(p, np.ones(p.n))
        assert _coarse_launches(p, lambda: p.gmg.apply(cv, dv)) == 0, over


def test_adjoint_gradient_identical():
    """the transposed multigrid of the adjoint solve uses the fused coarse
    cycle too; gradients are bit-identical"""
    import torch
    from ugcore_gb300 import adjoint, problems
    import ugcore_gb300 as ug
    out = []
    for levels in (0, -1):
        ctx = ug.Context(0)
        ctx.set_tuning(coarse_levels=levels)
        prob = adjoint.DifferentiableProblem(ctx, problems.config("c3", nref=5))
        m = torch.tensor(prob.m_top, device="cuda", requires_grad=True)
        f = torch.ones(prob.n, dtype=torch.float64, device="cuda")
        u = adjoint.fv1_solve(m, f, prob)
        (0.5 * (u ** 2).sum()).backward()
        out.append((u.detach().cpu().numpy(), m.grad.cpu().numpy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_reinitialisations_keep_bit_identity():
    """re-initialisations of the same multigrid (new coefficients; changed
    smoothing counts and cycle type) refresh the one-launch cycle's plan: its
    corrections stay bit-identical to the separate launches"""
    import torch
    import ugcore_gb300 as ug
    from ugcore_gb300 import adjoint, problems
    cfg = problems.config("c3", nref=5)
    pr, pf = [], []
    for levels, out in ((0, pr), (-1, pf)):
        ctx = ug.Context(0)
        ctx.set_tuning(coarse_levels=levels)
        out.append(adjoint.DifferentiableProblem(ctx, cfg))
    d = np.random.default_rng(5).uniform(-1.0, 1.0, pr[0].n)
    m0 = torch.tensor(pr[0].m_top, device="cuda")
    f = torch.ones(pr[0].n, dtype=torch.float64, device="cuda")
    for step, (nu1, nu2, cycle) in enumerate([(2, 2, 1), (2, 2, 1), (1, 3, 1), (3, 0, 1), (2, 2, 2), (2, 2, 1)]):
        res = []
        for p in (pr[0], pf[0]):
            p.gmg.set_num_presmooth(nu1)
            p.gmg.set_num_postsmooth(nu2)
            p.gmg.set_cycle_type(cycle)
            p.update(m0 * (1.0 + 0.05 * step), f)
            cv, dv = _apply(p, d)
            res.append(cv.numpy())
        assert np.array_equal(res[0], res[1]), (step, float(np.abs(res[0] - res[1]).max()))
