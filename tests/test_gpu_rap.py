"""Galerkin coarse operators (set_rap): the GPU's R A P against the oracle
(restated AddMultiplyOf, itself pinned bit for bit against ugcore's own
AddMultiplyOf) and against the fixtures ugcore's algebra wrote.

Bars: CRS pattern bit-exact; values 1e-13 relative to the row's largest
entry (the top-level operators agree to that bar, and the products are formed
in the reference's order with explicit rounding); GMG-preconditioned solves:
iteration count +-1, relative residual < 1e-10."""
import numpy as np
import pytest

from helpers import assert_crs_equal, load_golden, oracle_params

pytestmark = pytest.mark.gpu

CASES = [
    ("c0", dict(nref=4)),
    ("c1", dict(nref=3)),
    ("c2", dict(nref=2)),
    ("c4", dict(nref=2)),
]


def _problem(ctx, name, over):
    from ugcore_gb300 import problems
    cfg = problems.config(name, rap=True, **over)
    if name != "c2":
        cfg["precision"] = over.get("precision", "fp64")
    return cfg, problems.Problem(ctx, cfg)


@pytest.mark.parametrize("name,over", CASES)
def test_rap_levels_match_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    for l in range(p.hier.num_levels):
        assert_crs_equal(p.gmg.level_matrix(l), op.gmg_level_matrix(l), what="R A P level %d" % l)


@pytest.mark.parametrize("name,over", CASES + [("c1", dict(nref=4, precision="mixed")),
                                               ("c2", dict(nref=3, precision="mixed"))])
def test_rap_solve_matches_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    st = p.solve()
    assert st["converged"]
    assert st["defect"] / st["initial_defect"] < 1e-10
    op = oracle_lib.Problem(oracle_params(oracle_lib, dict(cfg, precision="fp64")))
    ref = op.solve()
    assert abs(st["steps"] - ref["steps"]) <= 1, (st["steps"], ref["steps"])
    x = p.x.numpy()
    tol = 1e-8 if cfg["precision"] == "fp64" else 1e-6
    assert np.abs(x - ref["x"]).max() <= tol * np.abs(ref["x"]).max()


@pytest.mark.parametrize("name", ["hex_2x2x2_r2_rap", "tet_4x4x4_r1_lognormal_rap", "hex_3x3x3_r1_convection_rap"])
def test_rap_against_ugcore_golden(ctx, name):
    """coarse operators computed by ugcore's own AddMultiplyOf"""
    from ugcore_gb300 import problems
    g = load_golden(name)
    e, mx, my, mz, nref, seed, ck, solver, vk, diff, pe = g["params"][:11]
    cfg = problems.config("golden", elem=["quad", "hex", "tet"][int(e)], mx=int(mx), my=int(my), mz=int(mz),
                          nref=int(nref), seed=int(seed),
                          coef={0: "const", 1: "lognormal", 3: "const"}[int(ck)], diffusion=diff,
                          vel="curl" if vk else None, solver="cg" if solver == 0 else "bicgstab", peclet=pe,
                          rap=True)
    p = problems.Problem(ctx, cfg)
    nl = int(g["nlev"])
    for l in range(nl):
        assert_crs_equal(p.gmg.level_matrix(l), (g["A%d_rowptr" % l], g["A%d_col" % l], g["A%d_val" % l]),
                         what="level %d vs ugcore AddMultiplyOf" % l)
    st = p.solve()
    assert abs(st["steps"] - int(g["steps"])) <= 1
    x = p.x.numpy()
    assert np.abs(x - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()


def test_rap_adjoint_matches_oracle(ctx, oracle_lib):
    """transposed multigrid with Galerkin coarse operators of A^T (c4
    convection, BiCGStab): lambda = A^-T g against the oracle"""
    cfg, p = _problem(ctx, "c4", dict(nref=2, rel_red=1e-12, maxit=400))
    p.solve()
    rng = np.random.default_rng(5)
    g = rng.standard_normal(p.n)
    st = p.adjoint_solve(g)
    assert st["converged"]
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg))
    ref = op.adjoint(g)
    assert ref["converged"]
    lam = p.lam.numpy()
    assert np.abs(lam - ref["lam"]).max() <= 1e-8 * np.abs(ref["lam"]).max()
    assert abs(st["steps"] - ref["steps"]) <= 1
