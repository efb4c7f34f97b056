"""Theta time stepping (ThetaTimeStep over the FV1 discretisation) on the GPU
against the oracle's restatement of the instationary assembly
(lib_disc/spatial_disc/elem_disc/elem_disc_assemble_util.h:1032-1225 with the
scalings of lib_disc/time_disc/theta_time_step_impl.h:120-240).

Bars: CRS pattern bit-exact; time-discrete operator values 1e-13 relative to
the row's largest entry; right-hand side 1e-13 relative to its largest entry;
multigrid coarse operators (M + theta dt A of each level) as the operator;
time loop: iterations per step within +-1 of the oracle's (+-2 for the
mixed-precision multigrid against the FP64 oracle) and the solution within
1e-8 (FP64) / 1e-6 (mixed precision) of it, relative to its maximum."""
import numpy as np
import pytest

from helpers import assert_crs_equal, oracle_params

pytestmark = pytest.mark.gpu

CASES = [
    ("c0", dict(nref=4)),
    ("c1", dict(nref=3)),
    ("c2", dict(nref=2, precision="fp64")),
    ("c4", dict(nref=2, precision="fp64")),
]


def _setup(ctx, orc, name, over):
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    p = problems.Problem(ctx, cfg)
    op = orc.Problem(oracle_params(orc, cfg), m_top=getattr(p, "m_top", None))
    return cfg, p, op


def _u_old(p, seed):
    u = np.random.default_rng(seed).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    u[bnd.astype(bool)] = 0.0
    return u


@pytest.mark.parametrize("theta", [1.0, 0.5])
@pytest.mark.parametrize("name,over", CASES)
def test_theta_system_matches_oracle(ctx, oracle_lib, name, over, theta):
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    dt = 0.02
    u_old = _u_old(p, 7)
    td = ug.ThetaTimeStep(p.disc, theta)
    td.prepare_step(ug.GPUVector(ctx, p.n).copy_from(u_old), 0.0, dt)
    assert td.future_time() == dt
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, p.n)
    td.assemble_linear(A, b)
    (rp, ci, va), ob = op.theta_system(theta, dt, u_old)
    assert_crs_equal(A.export_csr(), (rp, ci, va), what="M + theta dt A")
    assert np.abs(b.numpy() - ob).max() <= 1e-13 * np.abs(ob).max()
    # the jacobian entry point gives the same operator
    J = ug.GPUSparseMatrix(ctx)
    td.assemble_jacobian(J)
    assert_crs_equal(J.export_csr(), (rp, ci, va), what="jacobian")


@pytest.mark.parametrize("name,over", CASES)
def test_multigrid_levels_are_time_discrete(ctx, oracle_lib, name, over):
    """GeometricMultiGrid.set_discretization(ThetaTimeStep): every level's
    operator is that level's M + theta dt A"""
    import ugcore_gb300 as ug
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    theta, dt = 1.0, 0.05
    td = ug.ThetaTimeStep(p.disc, theta)
    u = ug.GPUVector(ctx, p.n)
    td.prepare_step(u, 0.0, dt)
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, p.n)
    td.assemble_linear(A, b)
    g = p._make_gmg(transposed=False)
    g.set_precision("fp64")
    g.set_discretization(td)
    g.init(A)
    for l in range(p.hier.num_levels):
        assert_crs_equal(g.level_matrix(l), op.theta_jacobian(l, theta, dt), what="level %d" % l)


@pytest.mark.parametrize("theta", [1.0, 0.5])
@pytest.mark.parametrize("name,over", CASES + [("c1", dict(nref=4, precision="mixed")),
                                               ("c2", dict(nref=3, precision="mixed"))])
def test_theta_steps_match_oracle(ctx, oracle_lib, name, over, theta):
    cfg, p, op = _setup(ctx, oracle_lib, name, over)
    dt, nsteps = 0.01, 4
    u0 = _u_old(p, 11)
    u, steps = p.theta_steps(theta, dt, nsteps, u0)
    ou, osteps = op.theta_steps(theta, dt, nsteps, u0)
    # the mixed-precision multigrid is a slightly different preconditioner
    # than the FP64 one the oracle applies, and each step starts from the
    # previous step's solution: its counts may drift by one more per run
    it_tol = 1 if cfg["precision"] == "fp64" else 2
    for s, (a, r) in enumerate(zip(steps, osteps)):
        assert abs(a - int(r)) <= it_tol, (s, steps, list(osteps))
    tol = 1e-8 if cfg["precision"] == "fp64" else 1e-6
    assert np.abs(u - ou).max() <= tol * np.abs(ou).max()


def test_stationary_solution_is_a_fixed_point(ctx):
    """from A u* = f every theta step returns u* (up to the solver's bar)"""
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c1", nref=3, rel_red=1e-12))
    p.solve()
    us = p.x.numpy()
    for theta in (1.0, 0.5):
        u, _ = p.theta_steps(theta, 0.1, 2, us)
        assert np.abs(u - us).max() <= 1e-8 * np.abs(us).max()
