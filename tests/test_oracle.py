"""Pins the CPU oracle: against ugcore's own golden data (the transpose test
log) and against fixtures produced by ugcore's own algebra (tests/golden),
plus geometry and generator properties.  CPU only."""
import os
import subprocess

import numpy as np
import pytest

from helpers import GOLDEN, assert_crs_equal, load_golden, oracle_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ---- ugcore tests/sm_transpose.cc + tests/ref/sm_transpose.out -------------
def _sm_test0(N, M):
    """matrix of test0() (tests/sm_transpose.cc:77-95)"""
    ent = {}
    for i in range(1, min(N, M)):
        ent[(i, i)] = 2.0
        ent[(i, i - 1)] = 1.0
        ent[(i - 1, i)] = 1.0
    if N > 6 and M > 6:
        ent[(5, 5)] = 0.0
        ent[(5, 0)] = 0.0
        ent[(1, 6)] = 1.0
    return ent, N, M


def _sm_test3(N):
    """matrix of test3() (tests/sm_transpose.cc:118-131)"""
    return {(i, j): float(i + j) for i in range(N) for j in range(N)}, N, N


def _to_crs(ent, N):
    rows = [[] for _ in range(N)]
    for (i, j), v in ent.items():
        rows[i].append((j, v))
    rp, ci, va = [0], [], []
    for r in rows:
        for j, v in sorted(r):
            ci.append(j)
            va.append(v)
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(va)


# (matrix, nnz of set_as_transpose_of, nnz of set_as_transpose_of2) from
# tests/ref/sm_transpose.out:1-30
SM_GOLDEN = [
    (lambda: _sm_test0(2, 2), 3, 3),
    (lambda: _sm_test0(10000, 10000), 29999, 29997),
    (lambda: _sm_test0(7, 10), 20, 18),
    (lambda: _sm_test0(10, 7), 20, 18),
    (lambda: _sm_test3(10), 100, 99),
    (lambda: _sm_test3(300), 90000, 89999),
]


@pytest.mark.parametrize("case", range(len(SM_GOLDEN)))
def test_transpose_matches_ugcore_golden(oracle_lib, case):
    make, nnz_keep, nnz_drop = SM_GOLDEN[case]
    ent, N, M = make()
    rp, ci, va = _to_crs(ent, N)
    assert oracle_lib.transpose_nnz(rp, ci, va, M, keep_zeros=True) == nnz_keep
    assert oracle_lib.transpose_nnz(rp, ci, va, M, keep_zeros=False) == nnz_drop


# ---- fixtures from ugcore's algebra (tests/golden/make_golden.py) ----------
GOLDEN_CASES = ["quad_2x2_r4", "hex_2x2x2_r2", "tet_4x4x4_r1_lognormal", "hex_3x3x3_r1_convection",
                "hex_2x2x2_r2_rap", "tet_4x4x4_r1_lognormal_rap", "hex_3x3x3_r1_convection_rap",
                "hex_3x3x3_r2_convection_restart2", "hex_3x3x3_r2_convection_minortho",
                "hex_3x3x3_r2_convection_restart4_minortho", "hex_2x2x2_r2_damped",
                "tet_4x4x4_r1_lognormal_damped"]


def _golden_problem(orc, g):
    e, mx, my, mz, nref, seed, ck, solver, vk, diff, pe = g["params"][:11]
    extra = {}
    if len(g["params"]) > 11:   # smoother, damp, nu1, nu2, maxit, rap
        sm, damp, nu1, nu2, maxit, rap = g["params"][11:17]
        extra = dict(smoother=int(sm), damp=float(damp), nu1=int(nu1), nu2=int(nu2), maxit=int(maxit), rap=int(rap))
    if len(g["params"]) > 17:   # BiCGStab restart period, minimal orthogonality
        extra.update(bicg_restart=int(g["params"][17]), bicg_min_ortho=float(g["params"][18]))
    if len(g["params"]) > 19:   # transfer damping (prolongation, restriction)
        extra.update(damp_prol=float(g["params"][19]), damp_res=float(g["params"][20]))
    p = orc.make_params(elem_type=int(e), mx=int(mx), my=int(my), mz=int(mz), nref=int(nref), seed=int(seed),
                        coef_kind=int(ck), solver=int(solver), vel_kind=int(vk), diffusion=diff, peclet=pe, **extra)
    return orc.Problem(p), bool(extra.get("rap", 0))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_reproduces_ugcore_algebra(oracle_lib, name):
    """level operators (re-assembled, or Galerkin R A P computed by ugcore's
    AddMultiplyOf in the *_rap cases), transfers, rhs, solution and defect
    history bit for bit"""
    g = load_golden(name)
    assert g is not None, "missing fixture " + name
    P, rap = _golden_problem(oracle_lib, g)
    nl = int(g["nlev"])
    assert P.nlev == nl
    for l in range(nl):
        got = P.gmg_level_matrix(l) if rap else P.matrix(l)
        ref = (g["A%d_rowptr" % l], g["A%d_col" % l], g["A%d_val" % l])
        assert_crs_equal(got, ref, rtol=0.0, what="level %d operator" % l)
    assert_crs_equal(P.transfer(nl - 1, 0), (g["P_rowptr"], g["P_col"], g["P_val"]), rtol=0.0, what="P")
    assert_crs_equal(P.transfer(nl - 1, 1), (g["R_rowptr"], g["R_col"], g["R_val"]), rtol=0.0, what="R")
    assert np.array_equal(P.rhs(), g["b"])
    s = P.solve(hist_cap=400)
    assert s["steps"] == int(g["steps"])
    assert np.array_equal(s["x"], g["x"])
    assert np.array_equal(s["history"], g["hist"])


def test_reference_driver_live(oracle_lib, tmp_path):
    """When the reference tree is present, rebuild the driver and compare live."""
    drv = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
    if not os.path.exists(drv):
        pytest.skip("oracle/_ref not built (no reference tree on this machine)")
    out = str(tmp_path / "r.bin")
    subprocess.check_call([drv, out, "1", "2", "2", "2", "2", "7", "0", "0", "0"], stdout=subprocess.DEVNULL)
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    R = mg.read_ref(out)
    P = oracle_lib.Problem(oracle_lib.make_params(elem_type=1, mx=2, my=2, mz=2, nref=2, seed=7))
    s = P.solve(hist_cap=100)
    assert s["steps"] == R["steps"] and np.array_equal(s["x"], R["x"])


# ---- geometry -------------------------------------------------------------
def test_fv1_geometry_unit_elements(oracle_lib):
    o = oracle_lib
    g = o.geometry(o.ORC_QUAD, [[0, 0], [1, 0], [1, 1], [0, 1]])
    assert np.allclose(g["vols"], 0.25)
    assert np.allclose(g["normals"], [[0.5, 0], [0, 0.5], [-0.5, 0], [0, -0.5]])
    hexc = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]
    g = o.geometry(o.ORC_HEX, hexc)
    assert np.allclose(g["vols"], 0.125)
    # every SCVF normal points from -> to with area 1/4
    c = np.array(hexc, float)
    for i in range(12):
        d = c[g["to"][i]] - c[g["frm"][i]]
        assert np.isclose(g["normals"][i] @ d, 0.25)
    g = o.geometry(o.ORC_TET, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
    assert np.allclose(g["vols"], 1.0 / 24.0, rtol=1e-14)


def test_fv1_gradients_reproduce_linear_functions(oracle_lib):
    """sum_sh u(x_sh) grad phi_sh = grad u for linear u, on distorted elements"""
    o = oracle_lib
    rng = np.random.default_rng(3)
    a = np.array([0.3, -1.2, 0.7])
    for et, base in [(o.ORC_QUAD, [[0, 0], [1, 0], [1, 1], [0, 1]]),
                     (o.ORC_HEX, [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1],
                                  [0, 1, 1]]),
                     (o.ORC_TET, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])]:
        X = np.array(base, float) + 0.1 * rng.standard_normal((len(base), len(base[0])))
        if et == o.ORC_HEX:
            X = np.array(base, float) * [1.0, 0.8, 1.3]   # trilinear maps keep linear exact on parallelepipeds
        g = o.geometry(et, X)
        dim = X.shape[1]
        u = X @ a[:dim]
        for ip in range(g["grads"].shape[0]):
            assert np.allclose(g["grads"][ip].T @ u, a[:dim], atol=1e-12)


# ---- seeded generators: product host code == oracle --------------------------
def test_field_generators_match_oracle(oracle_lib):
    import ctypes as C
    from ugcore_gb300 import fields
    L = oracle_lib.lib()
    L.orc_field_params.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_uint64, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.POINTER(C.c_double)]
    for dim, nm, kmax, seed in [(3, 64, 8.0, 1 ^ fields.COEF_SEED_XOR), (2, 32, 8.0, 5)]:
        k = np.zeros(nm * dim)
        ph = np.zeros(nm)
        amp = C.c_double()
        L.orc_field_params(0, dim, nm, kmax, seed, k.ctypes.data, ph.ctypes.data, None, C.byref(amp))
        f = fields.ScalarField(dim, nm, kmax, seed)
        assert np.array_equal(f.k.ravel(), k) and np.array_equal(f.phase, ph) and f.amp == amp.value
    nm = 16
    k, ph, c = np.zeros(nm * 3), np.zeros(nm), np.zeros(nm * 3)
    sc = C.c_double()
    L.orc_field_params(1, 3, nm, 2.0, 1 ^ fields.VEL_SEED_XOR, k.ctypes.data, ph.ctypes.data, c.ctypes.data,
                       C.byref(sc))
    f = fields.CurlField(nm, 2.0, 1 ^ fields.VEL_SEED_XOR)
    assert np.array_equal(f.k.ravel(), k) and np.array_equal(f.phase, ph) and np.array_equal(f.c.ravel(), c)
    assert f.scale == sc.value


def test_curl_field_is_divergence_free():
    from ugcore_gb300 import fields
    f = fields.CurlField(16, 2.0, 11)
    x = np.random.default_rng(0).random((50, 3))
    h = 1e-5
    div = sum((f(x + h * e)[:, i] - f(x - h * e)[:, i]) / (2 * h) for i, e in enumerate(np.eye(3)))
    assert np.abs(div).max() < 1e-6


def test_source_hash_matches_oracle(oracle_lib):
    from ugcore_gb300 import fields
    P = oracle_lib.Problem(oracle_lib.make_params(elem_type=0, nref=3, seed=42))
    assert np.array_equal(P.source(), fields.source_uniform(42, P.nv()))


# ---- solver-level properties of the oracle ----------------------------------
def test_tet_refinement_nests(oracle_lib):
    """every coarse Kuhn tet receives exactly 8 children when log K is coarsened"""
    o = oracle_lib
    P = o.Problem(o.make_params(elem_type=o.ORC_TET, mx=2, my=2, mz=2, nref=2, coef_kind=2),
                  m_top=np.ones(6 * 8 * 8 * 8 * 8))
    for l in range(P.nlev):
        assert np.allclose(np.log(P.coef(l)), 1.0)


def test_mcgs_oracle_converges(oracle_lib):
    o = oracle_lib
    P = o.Problem(o.make_params(elem_type=o.ORC_HEX, nref=3, smoother=1, damp=1.0))
    s = P.solve()
    assert s["converged"] and s["steps"] < 10


def test_ilu_smoother_oracle(oracle_lib):
    """multicolour ILU(0) smoother: the multigrid converges (Poisson CG) and
    needs no more BiCGStab steps than damped Jacobi on convection-diffusion"""
    o = oracle_lib
    P = o.Problem(o.make_params(elem_type=o.ORC_HEX, mx=2, my=2, mz=2, nref=3, smoother=3, damp=1.0))
    s = P.solve()
    assert s["converged"] and s["steps"] < 12
    C = o.Problem(o.make_params(elem_type=o.ORC_HEX, mx=3, my=3, mz=3, nref=2, smoother=3, damp=1.0, solver=1,
                                vel_kind=1, diffusion=1e-2, coef_kind=3))
    J = o.Problem(o.make_params(elem_type=o.ORC_HEX, mx=3, my=3, mz=3, nref=2, smoother=0, damp=0.6, solver=1,
                                vel_kind=1, diffusion=1e-2, coef_kind=3))
    sc, sj = C.solve(), J.solve()
    assert sc["converged"] and sj["converged"]
    assert sc["steps"] <= sj["steps"]


def test_symmetric_mcgs_is_symmetric_and_converges(oracle_lib):
    """the symmetric multicolour Gauss-Seidel smoother gives a symmetric
    multigrid preconditioner on a symmetric operator (M d1 . d2 = d1 . M d2
    away from the Dirichlet rows), as CG needs, and converges"""
    o = oracle_lib
    P = o.Problem(o.make_params(elem_type=o.ORC_QUAD, mx=2, my=2, nref=4, smoother=2, damp=1.0, nu1=2, nu2=2))
    s = P.solve()
    assert s["converged"] and s["steps"] < 12
    rng = np.random.default_rng(0)
    n = P.nv()
    rp, ci, va = P.matrix()
    bnd = np.array([va[rp[i]:rp[i + 1]][ci[rp[i]:rp[i + 1]] == i][0] == 1.0 and
                    np.count_nonzero(va[rp[i]:rp[i + 1]]) == 1 for i in range(n)])
    d1, d2 = rng.standard_normal(n), rng.standard_normal(n)
    d1[bnd] = d2[bnd] = 0.0
    a, b = P.apply_gmg(d1) @ d2, d1 @ P.apply_gmg(d2)
    assert abs(a - b) <= 1e-12 * abs(a)


def test_adjoint_oracle_matches_finite_differences(oracle_lib):
    o = oracle_lib
    rng = np.random.default_rng(1)
    base = o.make_params(elem_type=o.ORC_QUAD, nref=3, coef_kind=2, rel_red=1e-14, maxit=400)
    ne = 2 * 2 * 64
    m = 0.3 * rng.standard_normal(ne)
    P = o.Problem(base, m_top=m)
    u = P.solve()["x"]
    uobs = 0.5 * u
    lam = P.adjoint(u - uobs)["lam"]
    g = P.grad_logk(u, lam)
    J = lambda mm: 0.5 * np.sum((o.Problem(base, m_top=mm).solve()["x"] - uobs) ** 2)
    h = 1e-6
    for _ in range(3):
        d = rng.standard_normal(ne)
        fd = (J(m + h * d) - J(m - h * d)) / (2 * h)
        assert abs(fd - g @ d) <= 1e-6 * max(abs(fd), 1e-30) + 1e-12


# ---- theta time stepping (ThetaTimeStep over the FV1 discretisation) ------
def test_theta_mass_is_the_scv_volume(oracle_lib):
    """(M + theta dt A) - theta dt A = lumped mass: the SCV volumes, which sum
    to the volume of the unit square / cube on every interior row set"""
    orc = oracle_lib
    P = orc.Problem(orc.make_params(elem_type=orc.ORC_HEX, mx=2, my=2, mz=2, nref=2, seed=3))
    rp, ci, va = P.matrix()
    u0 = np.zeros(P.nv())
    dt, theta = 0.25, 1.0
    (rpt, cit, vat), _ = P.theta_system(theta, dt, u0)
    assert np.array_equal(rp, rpt) and np.array_equal(ci, cit)
    M = vat - theta * dt * va
    diag = np.zeros(P.nv())
    for i in range(P.nv()):
        for a in range(rp[i], rp[i + 1]):
            if ci[a] == i:
                diag[i] = M[a]
            else:
                assert abs(M[a]) <= 1e-15
    n = round(P.nv() ** (1 / 3))
    interior = np.array([0 < i % n < n - 1 and 0 < (i // n) % n < n - 1 and 0 < i // (n * n) < n - 1
                         for i in range(P.nv())])
    h = 1.0 / (n - 1)
    assert np.allclose(diag[interior], h ** 3, rtol=1e-12)


def test_theta_steps_keep_the_stationary_solution(oracle_lib):
    """from the stationary solution u* (A u* = f) every theta step returns u*"""
    orc = oracle_lib
    P = orc.Problem(orc.make_params(elem_type=orc.ORC_QUAD, mx=2, my=2, nref=4, seed=5, rel_red=1e-13, maxit=400))
    us = P.solve()["x"]
    for theta in (1.0, 0.5):
        u, steps = P.theta_steps(theta, 0.05, 3, us)
        assert np.abs(u - us).max() <= 1e-9 * np.abs(us).max()


def test_implicit_euler_approaches_the_stationary_solution(oracle_lib):
    orc = oracle_lib
    P = orc.Problem(orc.make_params(elem_type=orc.ORC_QUAD, mx=2, my=2, nref=3, seed=5, rel_red=1e-12, maxit=400))
    us = P.solve()["x"]
    u, steps = P.theta_steps(1.0, 10.0, 6, np.zeros(P.nv()))
    assert np.abs(u - us).max() <= 1e-6 * np.abs(us).max()
    assert all(s > 0 for s in steps)


def test_newton_line_search_paths(oracle_lib):
    """StandardLineSearch in the oracle's Newton (linear operator, accurate
    linear solves, so the full step lambda = 1 takes the defect to ~1e-10 and
    lambda = 2 leaves |d| unchanged): the default search is Newton without one;
    lambda_start = 2 is rejected (rho ~ 1 > 1 - 0.25 * 2) and lambda = 1
    accepted; check_all + accept_best evaluates every try and takes the best;
    accept_best after one rejected try takes it; without accept_best the search
    (and Newton) fails; max_defect caps the accepted defect."""
    orc = oracle_lib
    P = orc.Problem(orc.make_params(elem_type=orc.ORC_QUAD, mx=2, my=2, nref=3, seed=5, rel_red=1e-12, maxit=400))
    u0 = np.zeros(P.nv())
    ref = P.newton(u0, maxit=4, reduction=1e-9)
    assert ref[1] == 0 and ref[2] == 1
    r = P.newton(u0, maxit=4, reduction=1e-9, line_search={})
    assert r[1] == 0 and r[5] == ([1], [1.0])
    assert np.array_equal(r[0], ref[0]) and np.array_equal(r[4], ref[4])
    r = P.newton(u0, maxit=4, reduction=1e-9, line_search=dict(lambda_start=2.0))
    assert r[1] == 0 and r[5] == ([2], [1.0])
    assert np.abs(r[0] - ref[0]).max() <= 1e-14 * np.abs(ref[0]).max()
    r = P.newton(u0, maxit=4, reduction=1e-9,
                 line_search=dict(lambda_start=2.0, max_steps=3, accept_best=1, check_all=1))
    assert r[1] == 0 and r[5] == ([3], [1.0])
    r = P.newton(u0, maxit=2, reduction=1e-9, line_search=dict(lambda_start=2.0, max_steps=1, accept_best=1))
    assert r[1] == 1 and r[2] == 2 and r[5] == ([1, 1], [2.0, 2.0])
    assert all(abs(x / r[4][0] - 1.0) < 1e-6 for x in r[4])
    r = P.newton(u0, maxit=4, reduction=1e-9, line_search=dict(lambda_start=2.0, max_steps=1))
    assert r[1] == 3 and r[2] == 0 and r[5] == ([1], [2.0])
    r = P.newton(u0, maxit=4, reduction=1e-9,
                 line_search=dict(lambda_start=2.0, max_steps=1, accept_best=1, max_defect=0.5 * ref[4][0]))
    assert r[1] == 3 and r[5] == ([1], [2.0])


def test_backward_and_separate_smoothers_in_the_oracle(oracle_lib):
    """the oracle's post-smoother of its own: a post-smoother equal to the
    pre-smoother changes nothing; forward Gauss-Seidel before and backward
    after the coarse correction converges with CG like the symmetric
    smoother (+-2 steps); the backward sweep alone differs from the forward
    one"""
    o = oracle_lib
    base = dict(elem_type=o.ORC_HEX, mx=2, my=2, mz=2, nref=3, seed=3, smoother=1, damp=1.0)
    same = o.Problem(o.make_params(**base, post_smoother=1, post_damp=1.0)).solve()
    ref = o.Problem(o.make_params(**base)).solve()
    assert same["steps"] == ref["steps"] and np.array_equal(same["x"], ref["x"])
    st = o.Problem(o.make_params(**base, post_smoother=4, post_damp=1.0)).solve()
    sgs = o.Problem(o.make_params(**dict(base, smoother=2))).solve()
    assert st["converged"] and abs(st["steps"] - sgs["steps"]) <= 2
    P1 = o.Problem(o.make_params(**base))
    P4 = o.Problem(o.make_params(**dict(base, smoother=4)))
    d = np.random.default_rng(0).standard_normal(P1.nv())
    assert not np.array_equal(P1.apply_gmg(d), P4.apply_gmg(d))


NEWTON_GOLDEN = ["newton_quad_r4_ls", "newton_hex_r2_ls_accept_best", "newton_tet_lognormal_ls_check_all",
                 "newton_hex_theta_half", "newton_quad_plain"]


@pytest.mark.parametrize("name", NEWTON_GOLDEN)
def test_newton_matches_ugcore_newton_solver(oracle_lib, name):
    """The oracle's Newton loop (orc_prob_newton_ls) against ugcore's own
    NewtonSolver + StandardLineSearch + AssembledOperator + CG + StdConvCheck
    run on the same assembly and multigrid (tests/golden/make_newton_golden.py,
    oracle/ref_newton.cpp): the same Newton steps and return, the same
    accepted lambdas, the same total linear steps, the solution to 1e-12 and
    the final defect to 1e-9 relative.  Stationary and theta-step operators;
    plain steps, line searches that accept, that take the best of their
    tries, and that fail after checking all tries."""
    from ugcore_gb300 import fields
    o = oracle_lib
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    (elem, mx, my, mz, nref, seed, coef, diff, theta, dt, maxit, mind, red, ls_max, ls_start, ls_red, ls_best,
     ls_all, lin_red) = g["args"].tolist()
    P = o.Problem(o.make_params(elem_type=int(elem), mx=int(mx), my=int(my), mz=int(mz), nref=int(nref),
                                seed=int(seed), coef_kind=int(coef), diffusion=diff, rel_red=lin_red))
    nv = len(g["u"])
    u0 = np.array([0.1 * (2.0 * fields.hash_uniform(int(seed) + 7, i) - 1.0) for i in range(nv)])
    ls = None
    if ls_max > 0:
        ls = dict(max_steps=int(ls_max), lambda_start=ls_start, lambda_reduce=ls_red, accept_best=int(ls_best),
                  check_all=int(ls_all))
    out = P.newton(u0, maxit=int(maxit), min_defect=mind, reduction=red,
                   theta=None if theta < 0 else theta, dt=dt, u_old=None if theta < 0 else np.zeros(nv),
                   line_search=ls)
    u, rc, steps, lin, defs = out[:5]
    assert int(steps) == int(g["steps"])
    assert (rc == 0) == (int(g["rc"]) == 0)
    # ugcore counts the linear solve of a step whose line search fails, the
    # oracle's per-step list stops before that step
    if rc == 3:
        assert int(np.sum(lin)) < int(g["linear_steps"])
    else:
        assert int(np.sum(lin)) == int(g["linear_steps"])
    if ls is not None:
        lams = np.array(out[5][1])
        assert len(lams) == len(g["lambdas"])
        assert np.abs(lams - g["lambdas"]).max() <= 1e-9
    assert np.abs(u - g["u"]).max() <= 1e-12 * max(np.abs(g["u"]).max(), 1e-300)
    assert abs(defs[-1] - g["d1"]) <= 1e-9 * g["d1"] or (rc != 0 and int(steps) == 0)


THETA_GOLDEN = ["theta_quad_cn", "theta_hex_implicit_euler", "theta_tet_lognormal_explicit",
                "theta_quad_lognormal_0.7"]


@pytest.mark.parametrize("name", THETA_GOLDEN)
def test_theta_step_matches_ugcore_theta_time_step(oracle_lib, name):
    """The oracle's theta step against ugcore's own ThetaTimeStep
    (tests/golden/make_theta_golden.py, oracle/ref_theta.cpp): the time
    scalings ugcore passes to the domain discretisation are the restated
    ones, s_m = (1, -1), s_a = (theta dt, (1 - theta) dt), bit for bit; for
    every step of the series (advanced by ugcore's dense LU) the oracle's
    operator and right-hand side from the same previous solution, the defect
    of a perturbed iterate and the jacobian M + theta dt A equal what
    ThetaTimeStep assembled, bit for bit.  Crank-Nicolson, implicit and
    explicit Euler, theta = 0.7; quadrilaterals, hexahedra, lognormal
    tetrahedra."""
    from ugcore_gb300 import fields
    o = oracle_lib
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    elem, mx, my, mz, nref, seed, coef, theta, dt, ns = g["args"].tolist()
    P = o.Problem(o.make_params(elem_type=int(elem), mx=int(mx), my=int(my), mz=int(mz), nref=int(nref),
                                seed=int(seed), coef_kind=int(coef)))
    top = P.nlev - 1
    for s in range(int(ns)):
        sc = g["scales"][s]
        assert sc.tolist() == [1.0, theta * dt, -1.0, (1.0 - theta) * dt]
        u_old = g["u_old"][s]
        (_, _, va), b = P.theta_system(theta, dt, u_old)
        assert np.array_equal(va, g["A"][s]) and np.array_equal(b, g["b"][s]), s
        w = u_old + np.array([0.01 * (2.0 * fields.hash_uniform(int(seed) + 11, i) - 1.0) for i in range(len(u_old))])
        d = P.defect(w, theta=theta, dt=dt, u_old=u_old)
        assert np.array_equal(d, g["d"][s]), s
        _, _, jv = P.theta_jacobian(top, theta, dt)
        assert np.array_equal(jv, g["J"][s]), s


# ---- multicolour smoothers against ugcore's own smoothers in that order ----
# (tests/golden/make_smoother_golden.py: ug::ILU given the (colour, index)
# row ordering through ILU::set_ordering_algorithm, ilu.h:396; ug::GaussSeidel,
# SymmetricGaussSeidel, BackwardGaussSeidel with set_sor_relax on the system
# permuted to that order)
SMOOTHER_GOLDEN = ["smoothers_quad_r4", "smoothers_hex_r2", "smoothers_tet_lognormal_r1",
                   "smoothers_hex_convection_r1"]
# fixture key -> (oracle smoother kind, SOR factor / damping, base-solver steps);
# keys "lsK_..." are ugcore's LinearSolver with that smoother and
# StdConvCheck(K, 0, 0), as gmg:set_base_solver sets it
SMOOTHER_KEYS = {"ilu": (3, 1.0, 1), "gs_1.0": (1, 1.0, 1), "gs_1.3": (1, 1.3, 1), "sgs_1.0": (2, 1.0, 1),
                 "sgs_1.3": (2, 1.3, 1), "sgs_0.7": (2, 0.7, 1), "bgs_1.0": (4, 1.0, 1), "bgs_0.8": (4, 0.8, 1),
                 "jacobi_0.6": (0, 0.6, 1), "ls5_jacobi_0.6": (0, 0.6, 5), "ls2_gs_1.0": (1, 1.0, 2),
                 "ls3_sgs_1.3": (2, 1.3, 3), "ls3_bgs_0.8": (4, 0.8, 3), "ls4_ilu": (3, 1.0, 4)}


def smoother_golden_problem(orc, z, kind, relax, steps=1):
    """the oracle problem of a smoother fixture, the smoother as the base
    solver of a one-level cycle (one step from zero returns c = B d)"""
    elem = str(z["elem"])
    mx, my, mz, nref, seed, ck, vk, diffusion, peclet = z["params"]
    et = {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET}[elem]
    p = orc.make_params(elem_type=et, mx=int(mx), my=int(my), mz=int(mz), nref=int(nref), seed=int(seed),
                        coef_kind=int(ck), vel_kind=int(vk), diffusion=float(diffusion), peclet=float(peclet),
                        smoother=kind, damp=relax, base=int(nref), base_steps=steps)
    return orc.Problem(p)


@pytest.mark.parametrize("name", SMOOTHER_GOLDEN)
def test_multicolour_smoothers_are_ugcore_smoothers_in_that_order(oracle_lib, name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    for key, (kind, relax, steps) in SMOOTHER_KEYS.items():
        P = smoother_golden_problem(oracle_lib, z, kind, relax, steps)
        rp, ci, va = P.matrix()
        assert ci.size == int(z["nnz"])
        assert abs(np.abs(va).sum() - float(z["val_sum"])) <= 1e-13 * float(z["val_sum"])
        for d, c in zip(z["d"], z["c_" + key]):
            co = P.apply_gmg(d)
            # ugcore divides by U_ii where the ILU restatement multiplies by 1/U_ii
            assert np.abs(co - c).max() <= 5e-15 * np.abs(c).max(), key
