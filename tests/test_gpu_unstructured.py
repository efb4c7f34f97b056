"""Assembly and GMG solves on unstructured hierarchies (UGX coarse grids
refined regularly) on the GPU, against the oracle run on the same levels
(exported from the library: coordinates, elements, Dirichlet vertices,
parents).

Bars as for the structured grids: CRS pattern bit-exact, values 1e-13
relative to the row's largest entry, right-hand side 1e-13, P and R
bit-exact, FP64 GMG application 1e-12, iteration count +-1 and solution
1e-8 (FP64), relative residual < 1e-10 in FP64 for mixed precision."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, assert_crs_equal

pytestmark = pytest.mark.gpu

GRIDS = os.path.join(GOLDEN, "grids")
CASES = [
    ("square_tris", "Dirichlet", 4, "const"),
    ("square_quads", "Boundary", 4, "const"),
    ("cube_tets", "Bottom", 3, "const"),
    ("cube_tets", None, 3, "lognormal"),
    ("cube_hexes", "Boundary", 3, "lognormal"),
]


def _setup(ctx, orc, name, dirichlet, nref, coef, precision="fp64", smoother="jacobi"):
    import ugcore_gb300 as ug
    from ugcore_gb300 import fields
    hier = ug.UnstructuredHierarchy.from_ugx(ctx, os.path.join(GRIDS, name + ".ugx"), nref, dirichlet)
    assert not hier.structured
    disc = ug.DomainDiscretization(hier)
    seed = 3
    if coef == "const":
        disc.set_diffusion(1.0)
    else:
        disc.set_diffusion_field(fields.ScalarField(hier.dim, 64, 8.0, seed ^ fields.COEF_SEED_XOR), factor=2.0)
    disc.set_source_uniform(seed)
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, hier.num_vertices())
    disc.assemble_linear(A, b)
    gmg = ug.GeometricMultiGrid(disc)
    gmg.set_smoother({"jacobi": lambda: ug.Jacobi(0.6), "mcgs": lambda: ug.GaussSeidel(1.0),
                      "mcsgs": lambda: ug.SymmetricGaussSeidel(1.0), "ilu": lambda: ug.ILU(1.0)}[smoother]())
    gmg.set_num_presmooth(2)
    gmg.set_num_postsmooth(2)
    gmg.set_base_level(0)
    gmg.set_precision(precision)
    gmg.init(A)
    levels = []
    for l in range(hier.num_levels):
        x, e, bnd = hier.export(l)
        npar, par = hier.parents(l) if l > 0 else (None, None)
        levels.append((x, e, bnd, npar, par))
    et = {0: orc.ORC_QUAD, 1: orc.ORC_HEX, 2: orc.ORC_TET, 3: orc.ORC_TRI}[hier.elem_type]
    params = orc.make_params(elem_type=et, seed=seed, coef_kind=0 if coef == "const" else 1, coef_modes=64,
                             coef_kmax=8.0, solver=0, smoother=0, damp=0.6, nu1=2, nu2=2, cycle=1, base=0,
                             maxit=200, rel_red=1e-10, min_defect=1e-300)
    op = orc.Problem(params, levels=levels)
    return hier, disc, A, b, gmg, op


@pytest.mark.parametrize("name,dirichlet,nref,coef", CASES)
def test_unstructured_assembly_and_transfers(ctx, oracle_lib, name, dirichlet, nref, coef):
    hier, disc, A, b, gmg, op = _setup(ctx, oracle_lib, name, dirichlet, nref, coef)
    assert_crs_equal(A.export_csr(), op.matrix(), what="top operator")
    ob = op.rhs()
    assert np.abs(b.numpy() - ob).max() <= 1e-13 * np.abs(ob).max()
    for l in range(1, hier.num_levels):
        assert_crs_equal(gmg.level_matrix(l - 1), op.matrix(l - 1), what="level %d operator" % (l - 1))
        for which in (0, 1):
            assert_crs_equal(gmg.transfer(l, which), op.transfer(l, which), rtol=0.0,
                             what="%s level %d" % ("PR"[which], l))


@pytest.mark.parametrize("name,dirichlet,nref,coef", CASES)
def test_unstructured_gmg_and_solve(ctx, oracle_lib, name, dirichlet, nref, coef):
    import ugcore_gb300 as ug
    hier, disc, A, b, gmg, op = _setup(ctx, oracle_lib, name, dirichlet, nref, coef)
    n = hier.num_vertices()
    d = np.random.default_rng(0).standard_normal(n)
    d[hier.export()[2].astype(bool)] = 0.0
    c = ug.GPUVector(ctx, n)
    gmg.apply(c, ug.GPUVector(ctx, n).copy_from(d))
    ref = op.apply_gmg(d)
    assert np.abs(c.numpy() - ref).max() <= 1e-12 * np.abs(ref).max()
    solver = ug.CG(ctx)
    solver.set_preconditioner(gmg)
    solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
    solver.init(A)
    x = ug.GPUVector(ctx, n)
    assert solver.apply(x, b)
    st = solver.stats()
    rs = op.solve()
    assert abs(st["steps"] - rs["steps"]) <= 1, (st, rs["steps"])
    assert np.abs(x.numpy() - rs["x"]).max() <= 1e-8 * np.abs(rs["x"]).max()


@pytest.mark.parametrize("precision,smoother", [("mixed", "jacobi"), ("fp64", "mcgs"), ("fp64", "mcsgs"),
                                               ("fp64", "ilu"), ("mixed", "ilu")])
def test_unstructured_variants_converge(ctx, oracle_lib, precision, smoother):
    """mixed precision, the multicolour Gauss-Seidel variants and ILU(0)
    (greedy vertex colours) on the tetrahedral hierarchy: the FP64 residual
    reaches 1e-10"""
    import ugcore_gb300 as ug
    hier, disc, A, b, gmg, op = _setup(ctx, oracle_lib, "cube_tets", "Bottom", 3, "lognormal", precision, smoother)
    solver = ug.CG(ctx)
    solver.set_preconditioner(gmg)
    solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
    solver.init(A)
    x = ug.GPUVector(ctx, hier.num_vertices())
    assert solver.apply(x, b)
    r = ug.GPUVector(ctx, hier.num_vertices())
    A.axpy(r, 1.0, b, -1.0, x)
    assert r.norm() / b.norm() < 1e-10
    rs = op.solve()
    assert np.abs(x.numpy() - rs["x"]).max() <= 1e-7 * np.abs(rs["x"]).max()


def test_unstructured_matches_structured_on_the_same_mesh(ctx):
    """the 2 x 2 quadrilateral unit square given as arrays and refined by the
    unstructured builder solves the same discrete problem as the structured
    hierarchy (vertices matched by coordinates)"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config("c0", nref=4, precision="fp64")
    p = problems.Problem(ctx, cfg)
    st = p.solve()
    xs = p.x.numpy()
    cs, _, _ = p.hier.export()
    assert p.hier.structured
    X0 = np.array([[x, y] for y in (0, .5, 1) for x in (0, .5, 1)])
    quads = np.array([(0, 1, 4, 3), (1, 2, 5, 4), (3, 4, 7, 6), (4, 5, 8, 7)], np.int32)
    hier = ug.UnstructuredHierarchy.from_arrays(ctx, "quad", X0, quads, num_refinements=4)
    disc = ug.DomainDiscretization(hier)
    disc.set_diffusion(1.0)
    # vertices matched by coordinates; the structured problem's rhs carried over
    cu, _, _ = hier.export()
    key = lambda c: np.round(c * 1024).astype(np.int64) @ np.array([1, 4096])
    pos = {k: i for i, k in enumerate(key(cs))}
    perm = np.array([pos[k] for k in key(cu)])
    bs = p.b.numpy()
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, hier.num_vertices())
    disc.assemble_linear(A, b)
    b.copy_from(bs[perm])
    gmg = ug.GeometricMultiGrid(disc)
    gmg.set_smoother(ug.Jacobi(0.6))
    gmg.set_precision("fp64")
    gmg.init(A)
    solver = ug.CG(ctx)
    solver.set_preconditioner(gmg)
    solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
    solver.init(A)
    x = ug.GPUVector(ctx, hier.num_vertices())
    assert solver.apply(x, b)
    assert abs(solver.stats()["steps"] - st["steps"]) <= 1
    assert np.abs(x.numpy() - xs[perm]).max() <= 1e-8 * np.abs(xs).max()
    # and the operators agree entry by entry after the renumbering
    rp, ci, va = A.export_csr()
    import scipy.sparse as sp
    Au = sp.csr_matrix((va, ci, rp)).toarray()
    rps, cis, vas = p.A.export_csr()
    As = sp.csr_matrix((vas, cis, rps)).toarray()
    assert np.abs(Au - As[np.ix_(perm, perm)]).max() <= 1e-13 * np.abs(As).max()


def _levels(hier):
    out = []
    for l in range(hier.num_levels):
        x, e, bnd = hier.export(l)
        npar, par = hier.parents(l) if l > 0 else (None, None)
        out.append((x, e, bnd, npar, par))
    return out


def _oracle_for(orc, hier, seed=3, **kw):
    et = {0: orc.ORC_QUAD, 1: orc.ORC_HEX, 2: orc.ORC_TET, 3: orc.ORC_TRI}[hier.elem_type]
    params = orc.make_params(elem_type=et, seed=seed, coef_kind=1, coef_modes=64, coef_kmax=8.0, solver=0,
                             smoother=0, damp=0.6, nu1=2, nu2=2, cycle=1, base=0, maxit=200, rel_red=1e-10,
                             min_defect=1e-300, **kw)
    return orc.Problem(params, levels=_levels(hier))


@pytest.mark.parametrize("name,dirichlet", [("cube_tets", "Bottom"), ("square_tris", "Dirichlet")])
def test_unstructured_galerkin_coarse_operators(ctx, oracle_lib, name, dirichlet):
    """set_rap on an unstructured hierarchy: R A P per level against the
    oracle's restated AddMultiplyOf on the same levels, and the solve"""
    import ugcore_gb300 as ug
    hier, disc, A, b, _, _ = _setup(ctx, oracle_lib, name, dirichlet, 3, "lognormal")
    gmg = ug.GeometricMultiGrid(disc)
    gmg.set_smoother(ug.Jacobi(0.6))
    gmg.set_precision("fp64")
    gmg.set_rap(True)
    gmg.init(A)
    op = _oracle_for(oracle_lib, hier, rap=1)
    for l in range(hier.num_levels):
        assert_crs_equal(gmg.level_matrix(l), op.gmg_level_matrix(l), what="R A P level %d" % l)
    solver = ug.CG(ctx)
    solver.set_preconditioner(gmg)
    solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
    solver.init(A)
    x = ug.GPUVector(ctx, hier.num_vertices())
    assert solver.apply(x, b)
    rs = op.solve()
    assert abs(solver.stats()["steps"] - rs["steps"]) <= 1
    assert np.abs(x.numpy() - rs["x"]).max() <= 1e-8 * np.abs(rs["x"]).max()


def test_unstructured_adjoint_solve(ctx, oracle_lib):
    """transposed operator (Dirichlet rows reset) and transposed multigrid on
    the tetrahedral hierarchy against the oracle's adjoint solve"""
    import ugcore_gb300 as ug
    hier, disc, A, b, _, _ = _setup(ctx, oracle_lib, "cube_tets", "Bottom", 3, "lognormal")
    AT = disc.adjoint_operator(A, ug.GPUSparseMatrix(ctx))
    gmg = ug.GeometricMultiGrid(disc)
    gmg.set_smoother(ug.Jacobi(0.6))
    gmg.set_precision("fp64")
    gmg.set_transposed(True)
    gmg.init(AT)
    solver = ug.CG(ctx)
    solver.set_preconditioner(gmg)
    solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
    solver.init(AT)
    n = hier.num_vertices()
    g = np.random.default_rng(4).standard_normal(n)
    bnd = hier.export()[2].astype(bool)
    rhs = ug.GPUVector(ctx, n).copy_from(np.where(bnd, 0.0, g))
    lam = ug.GPUVector(ctx, n)
    assert solver.apply(lam, rhs)
    ref = _oracle_for(oracle_lib, hier).adjoint(g)
    assert abs(solver.stats()["steps"] - ref["steps"]) <= 1
    assert np.abs(lam.numpy() - ref["lam"]).max() <= 1e-8 * np.abs(ref["lam"]).max()


@pytest.mark.parametrize("theta", [1.0, 0.5])
def test_unstructured_theta_step(ctx, oracle_lib, theta):
    """time-discrete system of one theta step on the triangle hierarchy"""
    import ugcore_gb300 as ug
    hier, disc, A, b, _, _ = _setup(ctx, oracle_lib, "square_tris", "Dirichlet", 3, "lognormal")
    n = hier.num_vertices()
    u_old = np.random.default_rng(2).standard_normal(n)
    u_old[hier.export()[2].astype(bool)] = 0.0
    td = ug.ThetaTimeStep(disc, theta)
    td.prepare_step(ug.GPUVector(ctx, n).copy_from(u_old), 0.0, 0.01)
    At = ug.GPUSparseMatrix(ctx)
    bt = ug.GPUVector(ctx, n)
    td.assemble_linear(At, bt)
    (rp, ci, va), ob = _oracle_for(oracle_lib, hier).theta_system(theta, 0.01, u_old)
    assert_crs_equal(At.export_csr(), (rp, ci, va), what="M + theta dt A")
    assert np.abs(bt.numpy() - ob).max() <= 1e-13 * np.abs(ob).max()


@pytest.mark.parametrize("smoother", ["mcgs", "ilu"])
def test_unstructured_galerkin_with_colour_smoothers(ctx, oracle_lib, smoother):
    """Galerkin coarse operators of an unstructured hierarchy couple vertices
    that share no coarse element; the colour-ordered smoothers colour each
    operator's own graph, so the solve converges and is bitwise reproducible"""
    import ugcore_gb300 as ug
    hier, disc, A, b, _, _ = _setup(ctx, oracle_lib, "cube_tets", "Bottom", 3, "lognormal")
    xs = []
    for _ in range(2):
        gmg = ug.GeometricMultiGrid(disc)
        gmg.set_smoother(ug.GaussSeidel(1.0) if smoother == "mcgs" else ug.ILU(1.0))
        gmg.set_precision("fp64")
        gmg.set_rap(True)
        gmg.init(A)
        solver = ug.CG(ctx)
        solver.set_preconditioner(gmg)
        solver.set_convergence_check(ug.StdConvCheck(200, 1e-300, 1e-10))
        solver.init(A)
        x = ug.GPUVector(ctx, hier.num_vertices())
        assert solver.apply(x, b)
        xs.append(x.numpy())
    assert np.array_equal(xs[0], xs[1])
    rs = _oracle_for(oracle_lib, hier).solve()
    assert np.abs(xs[0] - rs["x"]).max() <= 1e-8 * np.abs(rs["x"]).max()


def test_unstructured_log_coefficients_and_adjoint_gradient(ctx, oracle_lib):
    """per-element K = exp(m) on the tetrahedral hierarchy (coarse m = mean of
    the element's children): every level's operator against the oracle, and
    dJ/dm of J = 0.5 |u|^2 (transposed solve + element gradient) against the
    oracle's adjoint and central finite differences (h = 1e-5, 1e-6 relative)"""
    import ugcore_gb300 as ug
    hier = ug.UnstructuredHierarchy.from_ugx(ctx, os.path.join(GRIDS, "cube_tets.ugx"), 3, "Bottom")
    ne, n = hier.num_elements(), hier.num_vertices()
    m = 0.5 * np.random.default_rng(8).standard_normal(ne)
    disc = ug.DomainDiscretization(hier)
    disc.set_log_diffusion(m)
    disc.set_source_uniform(5)
    A = ug.GPUSparseMatrix(ctx)
    b = ug.GPUVector(ctx, n)
    disc.assemble_linear(A, b)
    params = oracle_lib.make_params(elem_type=oracle_lib.ORC_TET, seed=5, coef_kind=2, solver=0, smoother=0,
                                    damp=0.6, maxit=400, rel_red=1e-13, min_defect=1e-300)
    op = oracle_lib.Problem(params, m_top=m, levels=_levels(hier))
    assert_crs_equal(A.export_csr(), op.matrix(), what="top operator")
    for l in range(hier.num_levels):
        Al = ug.GPUSparseMatrix(ctx)
        disc.assemble_jacobian(Al, l)
        assert_crs_equal(Al.export_csr(), op.matrix(l), what="level %d operator" % l)

    def solve(Amat, rhs, transposed=False):
        gmg = ug.GeometricMultiGrid(disc)
        gmg.set_smoother(ug.Jacobi(0.6))
        gmg.set_precision("fp64")
        gmg.set_transposed(transposed)
        gmg.init(Amat)
        s = ug.CG(ctx)
        s.set_preconditioner(gmg)
        s.set_convergence_check(ug.StdConvCheck(400, 1e-300, 1e-13))
        s.init(Amat)
        x = ug.GPUVector(ctx, n)
        assert s.apply(x, rhs)
        return x

    u = solve(A, b)
    AT = disc.adjoint_operator(A, ug.GPUSparseMatrix(ctx))
    bnd = hier.export()[2].astype(bool)
    g = np.where(bnd, 0.0, u.numpy())
    lam = solve(AT, ug.GPUVector(ctx, n).copy_from(g), transposed=True)
    grad = disc.grad_logk(u, lam)
    ref = op.grad_logk(op.solve()["x"], op.adjoint(g)["lam"])
    assert np.abs(grad - ref).max() <= 1e-9 * np.abs(ref).max()

    def J(mm):
        disc.set_log_diffusion(mm)
        Am = ug.GPUSparseMatrix(ctx)
        bm = ug.GPUVector(ctx, n)
        disc.assemble_linear(Am, bm)
        x = solve(Am, bm).numpy()
        return 0.5 * float(x @ x)

    rng = np.random.default_rng(9)
    h = 1e-5
    for _ in range(3):
        d = rng.standard_normal(ne)
        fd = (J(m + h * d) - J(m - h * d)) / (2 * h)
        assert abs(grad @ d - fd) <= 1e-6 * abs(fd), (grad @ d, fd)
