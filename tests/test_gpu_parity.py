"""GPU parity: the CUDA path against the oracle and against fixtures from
ugcore's own algebra, at sizes the oracle finishes in seconds.

Bars (stated by the benchmark spec for this path):
  CRS row pointers / columns bit-exact; matrix values 1e-13 relative (to the
  row's largest entry); transfers P, R bit-exact (their weights are exact);
  FP64 GMG application 1e-12 relative; solve: same iteration count +-1 and
  the GPU solution's relative residual < 1e-10 (plus the difference to the
  oracle solution stated per case); mixed precision: relative residual
  < 1e-10 in FP64 and error against the FP64 oracle solution reported.
"""
import os

import numpy as np
import pytest

from helpers import assert_crs_equal, load_golden, oracle_params

pytestmark = pytest.mark.gpu

SMALL = [
    ("c0", dict(nref=5)),
    ("c1", dict(nref=3)),
    ("c2", dict(nref=2, precision="fp64")),
    ("c3", dict(nref=4)),
    ("c4", dict(nref=2, precision="fp64")),
]


def _problem(ctx, name, over):
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    return cfg, problems.Problem(ctx, cfg)


def _oracle(orc, cfg, p):
    return orc.Problem(oracle_params(orc, cfg), m_top=getattr(p, "m_top", None))


def _rel_residual(p, x):
    import ugcore_gb300 as ug
    r = ug.GPUVector(p.ctx, p.n)
    xv = ug.GPUVector(p.ctx, p.n).copy_from(x)
    p.A.axpy(r, 1.0, p.b, -1.0, xv)
    return r.norm() / p.b.norm()


@pytest.mark.parametrize("name,over", SMALL)
def test_assembly_matches_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    op = _oracle(oracle_lib, cfg, p)
    assert_crs_equal(p.A.export_csr(), op.matrix(), what="top operator")
    b = p.b.numpy()
    ob = op.rhs()
    assert np.abs(b - ob).max() <= 1e-13 * np.abs(ob).max()


@pytest.mark.parametrize("name,over", SMALL)
def test_transfers_match_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    op = _oracle(oracle_lib, cfg, p)
    for l in range(1, p.hier.num_levels):
        for which in (0, 1):
            assert_crs_equal(p.gmg.transfer(l, which), op.transfer(l, which), rtol=0.0,
                             what="%s level %d" % ("PR"[which], l))


@pytest.mark.parametrize("name,over", SMALL)
def test_gmg_apply_matches_oracle(ctx, oracle_lib, name, over):
    import ugcore_gb300 as ug
    cfg, p = _problem(ctx, name, over)
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(0).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    c_ref = op.apply_gmg(d)
    dv = ug.GPUVector(ctx, p.n).copy_from(d)
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, dv)
    err = np.abs(cv.numpy() - c_ref).max() / np.abs(c_ref).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("name,over", SMALL)
def test_solve_matches_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    st = p.solve()
    op = _oracle(oracle_lib, cfg, p)
    ref = op.solve(hist_cap=400)
    assert st["converged"]
    assert abs(st["steps"] - ref["steps"]) <= 1, (st["steps"], ref["steps"])
    x = p.x.numpy()
    assert _rel_residual(p, x) < 1e-10
    assert np.abs(x - ref["x"]).max() <= 1e-8 * np.abs(ref["x"]).max()
    h = p.solver.history()
    n = min(len(h), len(ref["history"]))
    assert np.allclose(h[:n], ref["history"][:n], rtol=1e-6, atol=0)


@pytest.mark.parametrize("name,over", [("c1", dict(nref=3, precision="mixed")),
                                       ("c2", dict(nref=2)),
                                       ("c4", dict(nref=2))])
def test_mixed_precision_converges_to_fp64_oracle(ctx, oracle_lib, name, over):
    cfg, p = _problem(ctx, name, over)
    assert cfg["precision"] == "mixed"
    st = p.solve()
    ref = _oracle(oracle_lib, cfg, p).solve()
    x = p.x.numpy()
    assert st["converged"] and _rel_residual(p, x) < 1e-10
    # the FP32 preconditioner changes iterates, not the converged solution
    err = np.abs(x - ref["x"]).max() / np.abs(ref["x"]).max()
    assert err < 1e-7, err
    assert st["steps"] <= ref["steps"] + 3


@pytest.mark.parametrize("name,smoother", [("c1", "mcgs"), ("c1", "mcsgs"), ("c0", "mcsgs"), ("c4", "mcsgs"),
                                           ("c1", "ilu"), ("c0", "ilu"), ("c4", "ilu"), ("c2", "ilu")])
def test_mcgs_smoother_matches_oracle(ctx, oracle_lib, name, smoother):
    """multicolour Gauss-Seidel, its symmetric variant (forward, then
    backward colour sweep) and multicolour ILU(0): GMG application 1e-12,
    solve iterations +-1"""
    import ugcore_gb300 as ug
    over = dict(nref=3 if name != "c0" else 5, smoother=smoother, damp=1.0, precision="fp64")
    if name in ("c4", "c2"):
        over["nref"] = 2
    cfg, p = _problem(ctx, name, over)
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(1).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    c_ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - c_ref).max() <= 1e-12 * np.abs(c_ref).max()
    st = p.solve()
    ref = op.solve()
    assert abs(st["steps"] - ref["steps"]) <= 1
    assert np.abs(p.x.numpy() - ref["x"]).max() <= 1e-8 * np.abs(ref["x"]).max()


@pytest.mark.parametrize("name,pre,post", [("c1", ("mcgs", 1.0), ("mcbgs", 1.0)), ("c0", ("mcgs", 1.2), ("mcbgs", 0.8)),
                                           ("c4", ("mcbgs", 1.0), ("ilu", 0.9)), ("c1", ("ilu", 1.0), ("mcsgs", 1.1)),
                                           ("c2", ("mcsgs", 0.9), ("mcgs", 1.0))])
def test_separate_pre_and_post_smoothers_match_oracle(ctx, oracle_lib, name, pre, post):
    """set_presmoother / set_postsmoother (mg_solver.h:179-183): forward
    Gauss-Seidel before and backward Gauss-Seidel after the coarse
    correction, ILU with a Gauss-Seidel kind, each with its own SOR
    relaxation / ILU factor; GMG application 1e-12 against the oracle, solve
    iterations +-1"""
    import ugcore_gb300 as ug
    over = dict(nref=3 if name != "c0" else 5, smoother=pre[0], damp=pre[1], post_smoother=post[0],
                post_damp=post[1], precision="fp64")
    if name in ("c4", "c2"):
        over["nref"] = 2
    cfg, p = _problem(ctx, name, over)
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(2).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    c_ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - c_ref).max() <= 1e-12 * np.abs(c_ref).max()
    st = p.solve()
    ref = op.solve()
    assert abs(st["steps"] - ref["steps"]) <= 1
    assert np.abs(p.x.numpy() - ref["x"]).max() <= 1e-8 * np.abs(ref["x"]).max()


@pytest.mark.parametrize("name,over", [("c1", dict(nref=3)), ("c1", dict(nref=3, row_assembly=0)),
                                       ("c2", dict(nref=2)), ("c0", dict(nref=4))])
def test_seeded_source_equals_explicit_source(ctx, name, over):
    """the seeded source f_i = 2 u(seed, i) - 1 (splitmix64 hash, its 53-bit
    integer scaled by 2^-53 in integer arithmetic on the device) gives the
    bits of the same source passed as an array (computed here with Python's
    own conversion), on the row-wise and on the element assembly"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import fields, problems
    over = dict(over)
    mode = over.pop("row_assembly", None)
    cfg = problems.config(name, **over)
    c = ctx
    if mode is not None:
        c = ug.Context(0)
        c.set_tuning(row_assembly=mode)
    p = problems.Problem(c, cfg)
    b_seed = p.b.numpy()
    p.disc.set_source(fields.source_uniform(cfg["seed"], p.n))
    A2, b2 = ug.GPUSparseMatrix(c), ug.GPUVector(c, p.n)
    p.disc.assemble_linear(A2, b2)
    assert np.array_equal(b_seed.view(np.int64), b2.numpy().view(np.int64))


@pytest.mark.parametrize("name,over", [
    ("c1", dict(nref=3, base=1, base_steps=20)),
    ("c0", dict(nref=5, base=2, smoother="mcsgs", damp=1.0, base_steps=8)),
    ("c2", dict(nref=2, base=1, precision="fp64", base_steps=10)),
    ("c1", dict(nref=4, base=3, base_steps=30)),          # 17^3 = 4913 base unknowns: beyond the dense LU
    ("c0", dict(nref=3, base=3, base_steps=5)),           # top = base: the cycle is the base iteration
    ("c4", dict(nref=2, base=1, precision="fp64", smoother="ilu", damp=1.0, base_steps=6)),
])
def test_smoothing_base_solver_matches_oracle(ctx, oracle_lib, name, over):
    """set_base_solver with a fixed number of pre-smoother steps (ugcore's
    LinearSolver with StdConvCheck(k, 0, 0), unsuccessful end suppressed):
    GMG application 1e-12 against the oracle, solve iterations +-1, also on
    a base level beyond the dense LU's 4096 unknowns and with top = base"""
    import ugcore_gb300 as ug
    cfg, p = _problem(ctx, name, dict(over, base_solver="smoother"))
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(5).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    c_ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - c_ref).max() <= 1e-12 * np.abs(c_ref).max()
    if cfg["base"] < cfg["nref"]:
        st = p.solve()
        ref = op.solve()
        assert abs(st["steps"] - ref["steps"]) <= 1
        assert np.abs(p.x.numpy() - ref["x"]).max() <= 1e-8 * np.abs(ref["x"]).max()


def test_smoothing_base_solver_mixed_precision(ctx, oracle_lib):
    """the base iteration in the FP32 multigrid: the FP64 solve converges to
    the FP64 oracle's solution"""
    cfg, p = _problem(ctx, "c1", dict(nref=4, base=3, base_solver="smoother", base_steps=30, precision="mixed"))
    st = p.solve()
    ref = _oracle(oracle_lib, dict(cfg, precision="fp64"), p).solve()
    assert st["converged"] and abs(st["steps"] - ref["steps"]) <= 2
    assert np.abs(p.x.numpy() - ref["x"]).max() <= 1e-7 * np.abs(ref["x"]).max()


def test_dense_lu_base_limit_is_reported(ctx):
    """the dense LU refuses a base level above 4096 unknowns with a message"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    with pytest.raises(ug.UG4GBError) as e:
        problems.Problem(ctx, problems.config("c1", nref=4, base=3))
    assert "4096" in str(e.value)


def test_jacobi_combines_only_with_itself(ctx):
    """a Jacobi pre-smoother with a Gauss-Seidel post-smoother, or two Jacobi
    dampings, are refused at init with a message (the Jacobi smoother works
    on the column-scaled level operator)"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c0", nref=3))
    for post in (ug.GaussSeidel(1.0), ug.Jacobi(0.5)):
        g = ug.GeometricMultiGrid(p.disc)
        g.set_smoother(ug.Jacobi(0.6))
        g.set_postsmoother(post)
        with pytest.raises(ug.UG4GBError) as e:
            g.init(p.A)
        assert "Jacobi" in str(e.value)


@pytest.mark.parametrize("name", ["quad_2x2_r4", "hex_2x2x2_r2", "tet_4x4x4_r1_lognormal", "hex_3x3x3_r1_convection"])
def test_gpu_against_ugcore_algebra_golden(ctx, name):
    """fixtures written by ugcore's own SparseMatrix/Jacobi/LU/CG/BiCGStab"""
    from ugcore_gb300 import problems
    g = load_golden(name)
    e, mx, my, mz, nref, seed, ck, solver, vk, diff, pe = g["params"]
    cfg = problems.config("golden", elem=["quad", "hex", "tet"][int(e)], mx=int(mx), my=int(my), mz=int(mz),
                          nref=int(nref), seed=int(seed),
                          coef={0: "const", 1: "lognormal", 3: "const"}[int(ck)], diffusion=diff,
                          vel="curl" if vk else None, solver="cg" if solver == 0 else "bicgstab", peclet=pe)
    p = problems.Problem(ctx, cfg)
    nl = int(g["nlev"])
    assert_crs_equal(p.A.export_csr(), (g["A%d_rowptr" % (nl - 1)], g["A%d_col" % (nl - 1)],
                                        g["A%d_val" % (nl - 1)]), what="top operator vs ugcore")
    assert_crs_equal(p.gmg.transfer(nl - 1, 0), (g["P_rowptr"], g["P_col"], g["P_val"]), rtol=0.0, what="P")
    assert_crs_equal(p.gmg.transfer(nl - 1, 1), (g["R_rowptr"], g["R_col"], g["R_val"]), rtol=0.0, what="R")
    st = p.solve()
    assert abs(st["steps"] - int(g["steps"])) <= 1
    x = p.x.numpy()
    assert np.abs(x - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()


@pytest.mark.parametrize("name", ["hex_3x3x3_r2_convection_restart2", "hex_3x3x3_r2_convection_minortho",
                                  "hex_3x3x3_r2_convection_restart4_minortho"])
def test_bicgstab_restarts_against_ugcore_golden(ctx, name):
    """BiCGStab::set_restart / set_min_orthogonality: fixtures written by
    ugcore's own BiCGStab (with the oracle's multigrid); steps +-1, defect
    history 1e-6, solution 1e-8"""
    from ugcore_gb300 import problems
    g = load_golden(name)
    par = g["params"]
    cfg = problems.config("c4", nref=int(par[4]), precision="fp64", bicg_restart=int(par[17]),
                          bicg_min_ortho=float(par[18]))
    p = problems.Problem(ctx, cfg)
    st = p.solve()
    assert abs(st["steps"] - int(g["steps"])) <= 1, (st["steps"], int(g["steps"]))
    x = p.x.numpy()
    assert np.abs(x - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()
    h = p.solver.history()
    n = min(len(h), len(g["hist"]))
    assert np.allclose(h[:n], g["hist"][:n], rtol=1e-6, atol=0)


@pytest.mark.parametrize("name,golden", [("c1", "hex_2x2x2_r2_damped"), ("c2", "tet_4x4x4_r1_lognormal_damped")])
def test_transfer_damping_against_ugcore_golden(ctx, oracle_lib, name, golden):
    """StdTransfer::set_prolongation_damping / set_restriction_damping:
    against fixtures from ugcore's SparseMatrix axpy / apply_ignore_zero_rows
    with the damping factors (steps +-1, solution 1e-8), and the damped
    multigrid application against the oracle's to 1e-12; the exported P and R
    stay undamped"""
    import ugcore_gb300 as ug
    g = load_golden(golden)
    par = g["params"]
    cfg = dict(nref=int(par[4]), precision="fp64", damp_prol=float(par[19]), damp_res=float(par[20]))
    cfg, p = _problem(ctx, name, cfg)
    st = p.solve()
    assert abs(st["steps"] - int(g["steps"])) <= 1, (st["steps"], int(g["steps"]))
    assert np.abs(p.x.numpy() - g["x"]).max() <= 1e-8 * np.abs(g["x"]).max()
    top = p.hier.num_levels - 1
    assert_crs_equal(p.gmg.transfer(top, 0), (g["P_rowptr"], g["P_col"], g["P_val"]), rtol=0.0, what="P")
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(4).standard_normal(p.n)
    d[p.hier.export()[2].astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    # the FP32 multigrid with the same damping: converged, close to FP64
    _, pm = _problem(ctx, name, dict(cfg, precision="mixed"))
    sm = pm.solve()
    assert sm["converged"] and abs(sm["steps"] - st["steps"]) <= 2
    assert np.abs(pm.x.numpy() - p.x.numpy()).max() <= 1e-7 * np.abs(p.x.numpy()).max()


@pytest.mark.parametrize("name,over", [("c0", dict(nref=5)), ("c1", dict(nref=3)), ("c2", dict(nref=3)),
                                       ("c3", dict(nref=4)), ("c4", dict(nref=3))])
def test_row_assembly_matches_element_assembly(ctx, name, over):
    """structured levels: the row-wise assembly (per-class geometry, every
    value written once) and the element kernel give the same operator and
    rhs to 1e-13 of the row maximum on every level; the row-wise result is
    bit-reproducible"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    c2 = ug.Context(0)
    c2.set_tuning(row_assembly=False)
    p1 = problems.Problem(ctx, cfg)
    p2 = problems.Problem(c2, cfg)
    for l in range(p1.hier.num_levels):
        A1, A2 = ug.GPUSparseMatrix(ctx), ug.GPUSparseMatrix(c2)
        p1.disc.assemble_jacobian(A1, l)
        p2.disc.assemble_jacobian(A2, l)
        assert_crs_equal(A1.export_csr(), A2.export_csr(), what="level %d" % l)
        A3 = ug.GPUSparseMatrix(ctx)
        p1.disc.assemble_jacobian(A3, l)
        assert np.array_equal(A1.export_csr()[2], A3.export_csr()[2])
    b1, b2 = p1.b.numpy(), p2.b.numpy()
    assert np.abs(b1 - b2).max() <= 1e-13 * np.abs(b2).max()


@pytest.mark.parametrize("name,over", [("c0", dict(nref=4)), ("c1", dict(nref=3)),
                                       ("c1", dict(nref=2, elem="tet")), ("c3", dict(nref=3, coef="const"))])
def test_uniform_stencil_assembly_matches_rows(ctx, name, over):
    """one coefficient and no convection: the interior stencil gathered once
    and written to every interior row gives the bits of the row-wise kernel,
    operator and rhs, on every level"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    assert cfg["coef"] == "const" and cfg.get("vel", "none") in (None, "none")
    c2 = ug.Context(0)
    c2.set_tuning(row_assembly=1)
    p1 = problems.Problem(ctx, cfg)
    p2 = problems.Problem(c2, cfg)
    for l in range(p1.hier.num_levels):
        A1, A2 = ug.GPUSparseMatrix(ctx), ug.GPUSparseMatrix(c2)
        p1.disc.assemble_jacobian(A1, l)
        p2.disc.assemble_jacobian(A2, l)
        e1, e2 = A1.export_csr(), A2.export_csr()
        assert np.array_equal(e1[0], e2[0]) and np.array_equal(e1[1], e2[1])
        assert np.array_equal(e1[2].view(np.int64), e2[2].view(np.int64)), "level %d" % l
    assert np.array_equal(p1.b.numpy().view(np.int64), p2.b.numpy().view(np.int64))


@pytest.mark.parametrize("name,over", [("c2", dict(nref=2)), ("c4", dict(nref=2)), ("c3", dict(nref=4))])
def test_bitwise_reproducible(ctx, name, over):
    """assembly (coloured, no atomics), reductions and the solve give the same
    bits in every run"""
    import ugcore_gb300 as ug
    cfg, p = _problem(ctx, name, over)
    a1 = p.A.export_csr()[2]
    b1 = p.b.numpy()
    p.solve()
    x1 = p.x.numpy()
    A2 = ug.GPUSparseMatrix(ctx)
    b2 = ug.GPUVector(ctx, p.n)
    p.disc.assemble_linear(A2, b2)
    assert np.array_equal(a1, A2.export_csr()[2]) and np.array_equal(b1, b2.numpy())
    p.solve()
    assert np.array_equal(x1, p.x.numpy())


@pytest.mark.parametrize("name,over", [("c0", dict(nref=4)), ("c1", dict(nref=3)), ("c2", dict(nref=2)),
                                       ("c4", dict(nref=2)), ("c1", dict(nref=3, smoother="mcgs", damp=1.0)),
                                       ("c1", dict(nref=6, precision="mixed")), ("c2", dict(nref=5))])
def test_sell_and_diagonal_layouts_agree(ctx, name, over):
    """the automatic diagonal layout and SELL-32 give the same solve (the
    full-size mixed cases run the 4-rows-per-thread FP32 smoother on the top
    level).  The two layouts map rows to threads differently, so the fused
    (z, r) reduction sums in a different order: the iteration counts agree
    within the +-1 bar of the parity contract."""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    c2 = ug.Context(0)
    c2.set_operator_format("sell")
    p1 = problems.Problem(ctx, cfg)
    p2 = problems.Problem(c2, cfg)
    s1, s2 = p1.solve(), p2.solve()
    assert abs(s1["steps"] - s2["steps"]) <= 1
    assert s1["defect"] / s1["initial_defect"] < 1e-10 and s2["defect"] / s2["initial_defect"] < 1e-10
    x1, x2 = p1.x.numpy(), p2.x.numpy()
    tol = 1e-13 if cfg["precision"] == "fp64" else 1e-7
    assert np.abs(x1 - x2).max() <= tol * np.abs(x2).max()


@pytest.mark.parametrize("name,over", [("c1", dict(nref=4)), ("c2", dict(nref=3, precision="mixed")),
                                       ("c4", dict(nref=3))])
def test_programmatic_launch_is_bit_identical(ctx, name, over):
    """programmatic dependent launch changes scheduling only: the solve with
    it and without it is bit for bit the same"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    c2 = ug.Context(0)
    c2.set_tuning(pdl=False)
    p1 = problems.Problem(ctx, cfg)
    p2 = problems.Problem(c2, cfg)
    s1, s2 = p1.solve(), p2.solve()
    assert s1["steps"] == s2["steps"]
    assert np.array_equal(p1.x.numpy(), p2.x.numpy())


def test_edge_cases(ctx):
    """zero rhs (converged at step 0), single-level hierarchy (base == top),
    W-cycle, no pre-smoothing, base level above 0"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config("c0", nref=3)
    p = problems.Problem(ctx, cfg)
    p.b.set(0.0)
    st = p.solve()
    assert st["steps"] == 0 and np.all(p.x.numpy() == 0.0)
    # the same solve graph (its entry test skipped the loop) runs the loop for
    # a real right-hand side, and skips it again for zero
    p.disc.assemble_linear(p.A, p.b)
    st = p.solve()
    assert st["converged"] and st["steps"] > 1
    assert _rel_residual(p, p.x.numpy()) < 1e-10
    p.b.set(0.0)
    st = p.solve()
    assert st["steps"] == 0 and np.all(p.x.numpy() == 0.0)
    # BiCGStab ends in its prologue as well
    q = problems.Problem(ctx, problems.config("c4", nref=2, precision="fp64"))
    q.b.set(0.0)
    st = q.solve()
    assert st["steps"] == 0 and np.all(q.x.numpy() == 0.0)
    for over in [dict(nref=0), dict(nref=4, cycle=2), dict(nref=4, nu1=0), dict(nref=4, base=2),
                 dict(nref=4, nu1=1, nu2=3)]:
        cfg = problems.config("c0", **over)
        p = problems.Problem(ctx, cfg)
        st = p.solve()
        assert st["converged"], over
        assert _rel_residual(p, p.x.numpy()) < 1e-10


def test_error_reporting(ctx):
    import ugcore_gb300 as ug
    with pytest.raises(ug.UG4GBError):
        ug.StructuredHierarchy(ctx, "hex", 0, 1, 1, 1)
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c0", nref=3, maxit=2))
    with pytest.raises(ug.UG4GBError) as ei:
        p.solve()
    assert ei.value.code == -5
    g = ug.GeometricMultiGrid(p.disc)
    c = ug.GPUVector(ctx, p.n)
    with pytest.raises(ug.UG4GBError) as ei:
        g.apply(c, p.b)
    assert ei.value.code == -7


@pytest.mark.parametrize("smoother", ["mcsgs", "ilu"])
def test_smoothers_in_mixed_precision(ctx, smoother):
    """FP32 multigrid with the symmetric Gauss-Seidel / ILU smoother inside
    FP64 CG: relative residual < 1e-10, solution within 1e-7 of FP64"""
    cfg64, p64 = _problem(ctx, "c1", dict(nref=4, smoother=smoother, damp=1.0, precision="fp64"))
    cfg32, p32 = _problem(ctx, "c1", dict(nref=4, smoother=smoother, damp=1.0, precision="mixed"))
    s64, s32 = p64.solve(), p32.solve()
    assert s32["converged"] and s32["defect"] / s32["initial_defect"] < 1e-10
    assert abs(s32["steps"] - s64["steps"]) <= 2
    x64 = p64.x.numpy()
    assert np.abs(p32.x.numpy() - x64).max() <= 1e-7 * np.abs(x64).max()


@pytest.mark.parametrize("name,cycle,over", [("c1", 2, dict(nref=3)), ("c1", -1, dict(nref=3)),
                                             ("c2", -1, dict(nref=2, solver="bicgstab")), ("c0", 3, dict(nref=5)),
                                             ("c4", -1, dict(nref=2))])
def test_cycle_types_match_oracle(ctx, oracle_lib, name, cycle, over):
    """W-, F- (-1: the coarser level once as F, then once as V) and gamma = 3
    cycles (AssembledMultiGridCycle::lmgc, mg_solver_impl.hpp:2091-2134):
    GMG application 1e-12, solve iterations +-1.  The F-cycle is not a
    symmetric preconditioner, so its lognormal case runs BiCGStab, whose step
    count on this problem moves under rounding-level changes of the
    operator: the oracle alone needs 57 to 60 half steps when K is perturbed
    by 1e-16..1e-15 relative (wavenumbers scaled by 1 + k 1e-16, |k| <= 12);
    that case is held to 10% and to the solution (1e-8)"""
    import ugcore_gb300 as ug
    cfg, p = _problem(ctx, name, dict(over, cycle=cycle, precision="fp64"))
    op = _oracle(oracle_lib, cfg, p)
    d = np.random.default_rng(2).standard_normal(p.n)
    d[p.hier.export()[2].astype(bool)] = 0.0
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, ug.GPUVector(ctx, p.n).copy_from(d))
    ref = op.apply_gmg(d)
    assert np.abs(cv.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    st, rs = p.solve(), op.solve()
    if cfg["solver"] == "bicgstab" and cfg["coef"] == "lognormal":
        assert abs(st["steps"] - rs["steps"]) <= max(1, 0.1 * rs["steps"]), (st["steps"], rs["steps"])
        assert np.abs(p.x.numpy() - rs["x"]).max() <= 1e-8 * np.abs(rs["x"]).max()
    else:
        assert abs(st["steps"] - rs["steps"]) <= 1


@pytest.mark.parametrize("name", ["smoothers_quad_r4", "smoothers_hex_r2", "smoothers_tet_lognormal_r1",
                                  "smoothers_hex_convection_r1"])
def test_smoothers_are_ugcore_smoothers_in_that_order(ctx, name):
    """the GPU's multicolour ILU(0) and Gauss-Seidel smoothers against ugcore's
    own ILU (given the same (colour, index) row ordering) and GaussSeidel /
    SymmetricGaussSeidel / BackwardGaussSeidel with set_sor_relax (on the
    system permuted to that order) and Jacobi, alone and as a k-step
    LinearSolver base solver (tests/golden/make_smoother_golden.py): the
    smoother as the base solver of a one-level cycle returns c = B d"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    from helpers import GOLDEN
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    mx, my, mz, nref, seed, ck, vk, diffusion, peclet = z["params"]
    kinds = {"ilu": "ilu", "gs": "mcgs", "sgs": "mcsgs", "bgs": "mcbgs", "jacobi": "jacobi"}
    for key in ("ilu", "gs_1.0", "gs_1.3", "sgs_1.0", "sgs_1.3", "sgs_0.7", "bgs_1.0", "bgs_0.8", "jacobi_0.6",
                "ls5_jacobi_0.6", "ls2_gs_1.0", "ls3_sgs_1.3", "ls3_bgs_0.8", "ls4_ilu"):
        # "lsK_...": ugcore's LinearSolver with that smoother and StdConvCheck(K, 0, 0)
        parts = key.split("_")
        steps = int(parts.pop(0)[2:]) if parts[0].startswith("ls") else 1
        kind, relax = parts[0], float(parts[1]) if len(parts) > 1 else 1.0
        over = dict(elem=str(z["elem"]), mx=int(mx), my=int(my), mz=int(mz), nref=int(nref), seed=int(seed),
                    coef={0: "const", 1: "lognormal", 3: "const"}[int(ck)], diffusion=float(diffusion),
                    vel="curl" if int(vk) else None, peclet=float(peclet), smoother=kinds[kind], damp=relax,
                    base=int(nref), base_solver="smoother", base_steps=steps, precision="fp64")
        p = problems.Problem(ctx, problems.config("c0", **over))
        _, ci, va = p.A.export_csr()
        assert ci.size == int(z["nnz"])
        assert abs(np.abs(va).sum() - float(z["val_sum"])) <= 1e-12 * float(z["val_sum"])
        for d, c in zip(z["d"], z["c_" + key]):
            dv = ug.GPUVector(ctx, p.n).copy_from(d)
            cv = ug.GPUVector(ctx, p.n)
            p.gmg.apply(cv, dv)
            assert np.abs(cv.numpy() - c).max() <= 1e-12 * np.abs(c).max(), key
