"""Defect assembly and the Newton solver on the GPU against the oracle.

Defect: DomainDiscretization::assemble_defect (domain_disc_impl.h:648) and
ThetaTimeStep::assemble_defect, element by element (add_def_A_elem +
add_rhs_elem, elem_disc_assemble_util.h:578-690 / 713-860), Dirichlet
entries 0.  Bar: 1e-13 relative to the size of the terms that cancel,
max_i (|A||u| + |f|)_i (the GPU sums the elements of a vertex in colour order,
the oracle in element order).

Newton: NewtonSolver::apply (newton_impl.h:171-340, no line search) with the
GMG-preconditioned CG / BiCGStab as linear solver.  Bars: the same number of
Newton steps as the oracle, linear steps per Newton step within +-1, the
solution within 1e-8 of the oracle's (relative to its maximum), the start
defect within 1e-12 relative, and every later defect (the residual a linear
solve left) within a factor of 10 of the oracle's or below 1e-12 of the
start defect."""
import numpy as np
import pytest

from helpers import oracle_params

pytestmark = pytest.mark.gpu

CASES = [
    ("c0", dict(nref=4, precision="fp64")),
    ("c1", dict(nref=3, precision="fp64")),
    ("c2", dict(nref=2, precision="fp64")),
    ("c4", dict(nref=2, precision="fp64")),
]


def _setup(ctx, orc, name, over):
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    p = problems.Problem(ctx, cfg)
    op = orc.Problem(oracle_params(orc, cfg), m_top=getattr(p, "m_top", None))
    return cfg, p, op


def _random(p, seed):
    u = np.random.default_rng(seed).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    u[bnd.astype(bool)] = 0.0
    return u


def _scale(op, u, extra=None):
    import scipy.sparse as sp
    rp, ci, va = op.matrix()
    A = sp.csr_matrix((np.abs(va), ci, rp), shape=(len(rp) - 1, len(rp) - 1))
    s = A @ np.abs(u) + np.abs(op.rhs())
    if extra is not None:
        s = s + extra
    return s.max()


@pytest.mark.parametrize("name,over", CASES)
def test_stationary_defect_matches_oracle(ctx, oracle_lib, name, over):
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    u = _random(p, 3)
    d = ug.GPUVector(ctx, p.n)
    p.disc.assemble_defect(d, ug.GPUVector(ctx, p.n).copy_from(u))
    ref = op.defect(u)
    assert np.abs(d.numpy() - ref).max() <= 1e-13 * _scale(op, u)
    # the defect is A u - b: the assembled operator applied by the SpMV agrees
    r = ug.GPUVector(ctx, p.n)
    p.A.axpy(r, -1.0, p.b, 1.0, ug.GPUVector(ctx, p.n).copy_from(u))
    assert np.abs(d.numpy() - r.numpy()).max() <= 1e-13 * _scale(op, u)


@pytest.mark.parametrize("theta", [1.0, 0.5])
@pytest.mark.parametrize("name,over", CASES)
def test_theta_defect_matches_oracle(ctx, oracle_lib, name, over, theta):
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    dt = 0.03
    u_old, u = _random(p, 4), _random(p, 5)
    td = ug.ThetaTimeStep(p.disc, theta)
    td.prepare_step(ug.GPUVector(ctx, p.n).copy_from(u_old), 0.0, dt)
    d = ug.GPUVector(ctx, p.n)
    td.assemble_defect(d, ug.GPUVector(ctx, p.n).copy_from(u))
    ref = op.defect(u, theta=theta, dt=dt, u_old=u_old)
    assert np.abs(d.numpy() - ref).max() <= 1e-13 * _scale(op, u + u_old, np.abs(u) + np.abs(u_old))
    # consistency with the time-discrete linear system: d = (M + theta dt A) u - rhs
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, p.n)
    td.assemble_linear(A, b)
    r = ug.GPUVector(ctx, p.n)
    A.axpy(r, -1.0, b, 1.0, ug.GPUVector(ctx, p.n).copy_from(u))
    assert np.abs(d.numpy() - r.numpy()).max() <= 1e-13 * _scale(op, u + u_old, np.abs(u) + np.abs(u_old))


def test_adjust_solution_sets_dirichlet_values(ctx):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c1", nref=2))
    u = ug.GPUVector(ctx, p.n).copy_from(np.arange(p.n, dtype=np.float64) + 1.0)
    p.disc.adjust_solution(u)
    _, _, bnd = p.hier.export()
    x = u.numpy()
    assert np.all(x[bnd.astype(bool)] == 0.0)
    assert np.array_equal(x[~bnd.astype(bool)], (np.arange(p.n) + 1.0)[~bnd.astype(bool)])


def _newton(ctx, p, cfg):
    import ugcore_gb300 as ug
    lin = (ug.CG if cfg["solver"] == "cg" else ug.BiCGStab)(ctx)
    gmg = p._make_gmg(transposed=False)
    lin.set_preconditioner(gmg)
    lin.set_convergence_check(ug.StdConvCheck(cfg["maxit"], cfg["min_defect"], cfg["rel_red"]))
    nw = ug.NewtonSolver(ctx)
    nw.set_linear_solver(lin)
    nw.set_convergence_check(ug.StdConvCheck(6, 1e-50, 1e-12))
    return nw, gmg


def _compare(nw, u, ref):
    ou, orc_rc, osteps, ols, odefs = ref
    st = nw.stats()
    assert orc_rc == 0
    assert st["steps"] == osteps, (st, osteps)
    for a, b in zip(st["linear_steps"], ols):
        assert abs(a - int(b)) <= 1, (st["linear_steps"], list(ols))
    h = nw.history()
    assert len(h) == len(odefs)
    assert abs(h[0] - odefs[0]) <= 1e-12 * odefs[0]
    floor = 1e-12 * odefs[0]
    for a, b in zip(h[1:], odefs[1:]):
        assert (a <= max(10 * b, floor) and b <= max(10 * a, floor)), (list(h), list(odefs))
    assert np.abs(u - ou).max() <= 1e-8 * np.abs(ou).max()


@pytest.mark.parametrize("name,over", CASES + [("c1", dict(nref=4, precision="mixed"))])
def test_newton_stationary_matches_oracle(ctx, oracle_lib, name, over):
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    cfg = dict(cfg, rel_red=1e-8)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    u0 = _random(p, 6)
    nw, _ = _newton(ctx, p, cfg)
    nw.init(ug.AssembledOperator(p.disc))
    u = ug.GPUVector(ctx, p.n).copy_from(u0)
    assert nw.apply(u)
    _compare(nw, u.numpy(), op.newton(u0, maxit=6, reduction=1e-12))


@pytest.mark.parametrize("theta", [1.0, 0.5])
@pytest.mark.parametrize("name,over", [("c1", dict(nref=3, precision="fp64")), ("c4", dict(nref=2, precision="fp64"))])
def test_newton_theta_step_matches_oracle(ctx, oracle_lib, name, over, theta):
    """one time step solved by Newton on the time-discrete operator, the
    multigrid levels assembled as the step's jacobian"""
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    cfg = dict(cfg, rel_red=1e-8)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    dt = 0.02
    u_old = _random(p, 7)
    td = ug.ThetaTimeStep(p.disc, theta)
    td.prepare_step(ug.GPUVector(ctx, p.n).copy_from(u_old), 0.0, dt)
    nw, gmg = _newton(ctx, p, cfg)
    gmg.set_discretization(td)
    nw.init(ug.AssembledOperator(td))
    u = ug.GPUVector(ctx, p.n).copy_from(u_old)
    assert nw.apply(u)
    _compare(nw, u.numpy(), op.newton(u_old, maxit=6, reduction=1e-12, theta=theta, dt=dt, u_old=u_old))


def test_newton_not_converged_is_reported(ctx):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config("c1", nref=3, rel_red=1e-2)
    p = problems.Problem(ctx, cfg)
    nw, _ = _newton(ctx, p, cfg)
    nw.set_convergence_check(ug.StdConvCheck(1, 1e-50, 1e-12))
    nw.init(ug.AssembledOperator(p.disc))
    u = ug.GPUVector(ctx, p.n)
    assert nw.apply(u, raise_on_failure=False) is False
    assert nw.stats()["steps"] == 1
    with pytest.raises(ug.UG4GBError):
        nw.apply(u)


LS_CASES = [
    (dict(lambda_start=2.0), "rejects the overshooting lambda = 2, accepts lambda = 1"),
    (dict(lambda_start=2.0, max_steps=3, accept_best=1, check_all=1), "evaluates all three tries, takes the best"),
    (dict(lambda_start=1.0, lambda_reduce=0.25, alpha=0.6), "sufficient descent 0.6"),
]


@pytest.mark.parametrize("ls", [c[0] for c in LS_CASES])
@pytest.mark.parametrize("name,over", [("c1", dict(nref=3, precision="fp64")), ("c4", dict(nref=2, precision="fp64")),
                                       ("c1", dict(nref=3, precision="mixed"))])
def test_newton_line_search_matches_oracle(ctx, oracle_lib, name, over, ls):
    """Newton with StandardLineSearch (inexact linear solves to 1e-8, so
    several Newton steps): the same tries and accepted lambdas per step as the
    oracle, and the same solution"""
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    cfg = dict(cfg, rel_red=1e-8)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    u0 = _random(p, 6)
    nw, _ = _newton(ctx, p, cfg)
    s = ug.StandardLineSearch(ls.get("max_steps", 10), ls["lambda_start"], ls.get("lambda_reduce", 0.5),
                              bool(ls.get("accept_best", 0)), bool(ls.get("check_all", 0)))
    s.set_suff_descent_factor(ls.get("alpha", 0.25))
    nw.set_line_search(s)
    nw.init(ug.AssembledOperator(p.disc))
    u = ug.GPUVector(ctx, p.n).copy_from(u0)
    assert nw.apply(u)
    ref = op.newton(u0, maxit=6, reduction=1e-12, line_search=ls)
    _compare(nw, u.numpy(), ref[:5])
    tries, lams = nw.line_search_history()
    assert tries == ref[5][0] and lams == ref[5][1], (tries, lams, ref[5])


def test_newton_line_search_on_a_theta_step(ctx, oracle_lib):
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, "c1", dict(nref=3, precision="fp64"))
    cfg = dict(cfg, rel_red=1e-8)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    dt, theta = 0.02, 0.5
    u_old = _random(p, 7)
    td = ug.ThetaTimeStep(p.disc, theta)
    td.prepare_step(ug.GPUVector(ctx, p.n).copy_from(u_old), 0.0, dt)
    nw, gmg = _newton(ctx, p, cfg)
    gmg.set_discretization(td)
    nw.set_line_search(ug.StandardLineSearch(lambda_start=2.0))
    nw.init(ug.AssembledOperator(td))
    u = ug.GPUVector(ctx, p.n).copy_from(u_old)
    assert nw.apply(u)
    ref = op.newton(u_old, maxit=6, reduction=1e-12, theta=theta, dt=dt, u_old=u_old,
                    line_search=dict(lambda_start=2.0))
    _compare(nw, u.numpy(), ref[:5])
    assert nw.line_search_history() == (ref[5][0], ref[5][1])


def test_newton_line_search_failures(ctx, oracle_lib):
    """without accept_best a search whose tries all fail ends Newton
    (NewtonSolver::apply returns false); with accept_best the best try is
    taken, and max_defect caps it"""
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, "c1", dict(nref=3, precision="fp64"))
    u0 = _random(p, 6)
    nw, _ = _newton(ctx, p, cfg)
    nw.init(ug.AssembledOperator(p.disc))
    nw.set_line_search(ug.StandardLineSearch(max_steps=1, lambda_start=2.0))
    u = ug.GPUVector(ctx, p.n).copy_from(u0)
    assert nw.apply(u, raise_on_failure=False) is False
    assert nw.line_search_history() == ([1], [2.0])
    assert nw.stats()["steps"] == 0
    with pytest.raises(ug.UG4GBError, match="line search"):
        nw.apply(ug.GPUVector(ctx, p.n).copy_from(u0))
    ls = ug.StandardLineSearch(max_steps=1, lambda_start=2.0, accept_best=True)
    nw.set_line_search(ls)
    nw.set_convergence_check(ug.StdConvCheck(2, 1e-50, 1e-12))
    u = ug.GPUVector(ctx, p.n).copy_from(u0)
    assert nw.apply(u, raise_on_failure=False) is False
    ref = op.newton(u0, maxit=2, reduction=1e-12, line_search=dict(max_steps=1, lambda_start=2.0, accept_best=1))
    assert ref[1] == 1 and nw.line_search_history() == ref[5] == ([1, 1], [2.0, 2.0])
    h = nw.history()
    assert np.allclose(h, ref[4], rtol=1e-6)
    ls.set_maximum_defect(0.5 * h[0])
    nw.set_line_search(ls)
    with pytest.raises(ug.UG4GBError, match="defect-limit"):
        nw.apply(ug.GPUVector(ctx, p.n).copy_from(u0))
    nw.set_line_search(None)
    nw.set_convergence_check(ug.StdConvCheck(6, 1e-50, 1e-12))
    assert nw.apply(ug.GPUVector(ctx, p.n).copy_from(u0))
    assert nw.line_search_history() == ([], [])
    with pytest.raises(ug.UG4GBError):
        nw.set_line_search(ug.StandardLineSearch(max_steps=0))


@pytest.mark.parametrize("freq,expected", [(0, None), (1, None), (2, "half"), (100, 1)])
def test_newton_reassemble_jacobian_frequency(ctx, oracle_lib, freq, expected):
    """set_reassemble_J_freq: the jacobian is assembled in steps 0, k, 2k, ...
    only; the FV1 operator is linear, so the reused jacobian is the same
    matrix and the iterates are bit-identical to reassembling every step"""
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, "c1", dict(nref=3, precision="fp64"))
    cfg = dict(cfg, rel_red=1e-6)
    u0 = _random(p, 6)
    res = []
    for f in (0, freq):
        nw, _ = _newton(ctx, p, cfg)
        nw.set_reassemble_J_freq(f)
        nw.init(ug.AssembledOperator(p.disc))
        u = ug.GPUVector(ctx, p.n).copy_from(u0)
        assert nw.apply(u)
        res.append((u.numpy(), nw.history(), nw.stats()["steps"], nw.num_jacobian_assemblies()))
    (u_a, h_a, s_a, n_a), (u_b, h_b, s_b, n_b) = res
    assert s_a >= 2 and s_a == s_b and n_a == s_a
    assert np.array_equal(u_a.view(np.int64), u_b.view(np.int64)) and np.array_equal(h_a, h_b)
    if expected is None:
        assert n_b == s_b
    elif expected == "half":
        assert n_b == (s_b + 1) // 2
    else:
        assert n_b == 1
    with pytest.raises(ug.UG4GBError):
        nw.set_reassemble_J_freq(-1)
