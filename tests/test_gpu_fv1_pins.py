"""The GPU's FV1 operators pinned outside the oracle's restatement (see
tests/test_fv1_pins.py for the CPU side and the derivations).

  - fixture meshes (distorted quadrilaterals, hexahedra, tetrahedra,
    triangles; lognormal K per element; a 3D Fourier velocity field): the
    GPU operator equals the one assembled from ugcore's own FV1Geometry and
    ConvectionShapesFullUpwind, with and without convection;
  - simplices: the GPU diffusion operator on refined distorted meshes equals
    the P1 finite-element stiffness;
  - uniform quadrilaterals / hexahedra: interior rows are the closed-form
    box stencils;
  - full upwind: with a constant velocity v >= 0 on uniform hexahedra the
    convective part of an interior row is the first-order upwind difference
    h^2 (v_x (u_i - u_{i-x}) + v_y (u_i - u_{i-y}) + v_z (u_i - u_{i-z}));
    with the seeded curl field it conserves (column sums 0) and has
    off-diagonals <= 0 and diagonals >= 0.
Values 1e-13 relative to the row's largest entry.
"""
import types

import numpy as np
import pytest

from test_fv1_pins import FIX, _assert_rows, check_box_stencil

pytestmark = pytest.mark.gpu


def _dense(A, n):
    rp, ci, va = A.export_csr()
    D = np.zeros((n, n))
    D[np.repeat(np.arange(n), np.diff(rp)), ci] = va
    return D


def _field(k, c, phase, scale):
    k = np.atleast_2d(np.asarray(k, np.float64))
    return types.SimpleNamespace(k=k, c=np.atleast_2d(np.asarray(c, np.float64)),
                                 phase=np.atleast_1d(np.asarray(phase, np.float64)), nmodes=k.shape[0], scale=1.0)


def _assemble(ctx, hier, logk, vel=None):
    import ugcore_gb300 as ug
    disc = ug.DomainDiscretization(hier)
    disc.set_log_diffusion(logk)
    if vel is not None:
        disc.set_velocity_field(vel, vel.user_scale)
        disc.set_upwind("full")
    A = ug.GPUSparseMatrix(ctx)
    disc.assemble_jacobian(A)
    return A, disc


@pytest.mark.parametrize("t", ["quad", "hex", "tet", "tri"])
def test_gpu_operator_matches_ugcore_geometry_on_fixture_meshes(ctx, t):
    import ugcore_gb300 as ug
    fx = np.load(FIX)
    coords, elems, logk = fx["m_%s_coords" % t], fx["m_%s_elems" % t], fx["m_%s_logK" % t]
    hier = ug.UnstructuredHierarchy.from_arrays(ctx, t, coords, elems, num_refinements=0)
    c2, _, bnd = hier.export()
    assert np.array_equal(c2, coords)
    n = len(coords)
    A, _ = _assemble(ctx, hier, logk)
    _assert_rows(_dense(A, n), fx["m_%s_A_diffusion" % t], bnd)
    if coords.shape[1] == 3:
        vel = _field(fx["m_%s_vel_k" % t], fx["m_%s_vel_c" % t], fx["m_%s_vel_phase" % t], 1.0)
        vel.user_scale = float(fx["m_%s_vel_scale" % t])
        Av, _ = _assemble(ctx, hier, logk, vel)
        _assert_rows(_dense(Av, n), fx["m_%s_A" % t], bnd)


def _p1_stiffness_sparse(coords, elems, K):
    import scipy.sparse as sp
    n, dim = coords.shape
    X = coords[elems]                                  # ne x (dim+1) x dim
    D = np.transpose(X[:, 1:] - X[:, :1], (0, 2, 1))   # ne x dim x dim, columns = edges
    vol = np.abs(np.linalg.det(D)) / (2.0 if dim == 2 else 6.0)
    B = np.concatenate([-np.ones((dim, 1)), np.eye(dim)], axis=1)      # d(lambda)/d(ref coords)
    G = np.linalg.solve(np.transpose(D, (0, 2, 1)), np.broadcast_to(B, (len(elems), dim, dim + 1)))
    G = np.transpose(G, (0, 2, 1))                     # ne x (dim+1) x dim
    loc = (K * vol)[:, None, None] * np.einsum("eid,ejd->eij", G, G)
    rows = np.repeat(elems, dim + 1, axis=1).ravel()
    cols = np.tile(elems, (1, dim + 1)).ravel()
    return sp.csr_matrix((loc.ravel(), (rows, cols)), shape=(n, n))


@pytest.mark.parametrize("t", ["tet", "tri"])
def test_gpu_box_method_equals_p1_fem_on_refined_distorted_simplices(ctx, t):
    import ugcore_gb300 as ug
    fx = np.load(FIX)
    hier = ug.UnstructuredHierarchy.from_arrays(ctx, t, fx["m_%s_coords" % t], fx["m_%s_elems" % t],
                                                num_refinements=2)
    coords, elems, bnd = hier.export()
    m = np.random.default_rng(5).standard_normal(len(elems))
    A, disc = _assemble(ctx, hier, m)
    K = disc.coefficients()
    np.testing.assert_allclose(K, np.exp(m), rtol=1e-15)
    S = _p1_stiffness_sparse(coords, elems, K)
    rp, ci, va = A.export_csr()
    inner = np.flatnonzero(~bnd.astype(bool))
    for r in inner:
        srow = S.getrow(r)
        ref = dict(zip(srow.indices.tolist(), srow.data.tolist()))
        got = dict(zip(ci[rp[r]:rp[r + 1]].tolist(), va[rp[r]:rp[r + 1]].tolist()))
        assert set(ref) <= set(got)
        scale = max(abs(v) for v in ref.values())
        for c, v in got.items():
            assert abs(v - ref.get(c, 0.0)) <= 1e-13 * scale, (r, c, v, ref.get(c, 0.0))


@pytest.mark.parametrize("name,nref", [("c0", 4), ("c1", 3)])
def test_gpu_uniform_grids_give_closed_form_box_stencils(ctx, name, nref):
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config(name, nref=nref))
    rp, ci, va = p.A.export_csr()
    nx = 2 * (1 << nref) + 1
    check_box_stencil(rp, ci, va, nx, 2 if name == "c0" else 3, 1.0 / (nx - 1))


def _hex_problem(ctx, nref, vel):
    import ugcore_gb300 as ug
    hier = ug.StructuredHierarchy(ctx, "hex", 2, 2, 2, nref)
    disc = ug.DomainDiscretization(hier)
    disc.set_diffusion(1e-2)
    if vel is not None:
        disc.set_velocity_field(vel, vel.user_scale)
        disc.set_upwind("full")
    A = ug.GPUSparseMatrix(ctx)
    disc.assemble_jacobian(A)
    return hier, A


def test_gpu_full_upwind_with_constant_velocity_is_first_order_upwind(ctx):
    """v = (0.3, 0.5, 0.7) everywhere (one Fourier mode with k = 0 and phase
    -pi/2): convective part of interior rows = h^2 (v_x + v_y + v_z) on the
    diagonal and -h^2 v_d at the upstream neighbour along axis d"""
    nref = 2
    v = np.array([0.3, 0.5, 0.7])
    vel = _field([[0.0, 0.0, 0.0]], [v], [-np.pi / 2], 1.0)
    vel.user_scale = 1.0
    hier, Av = _hex_problem(ctx, nref, vel)
    _, A0 = _hex_problem(ctx, nref, None)
    n = hier.num_vertices()
    C = _dense(Av, n) - _dense(A0, n)
    nx = 2 * (1 << nref) + 1
    h = 1.0 / (nx - 1)
    checked = 0
    for r in range(n):
        i, j, k = r % nx, (r // nx) % nx, r // (nx * nx)
        if min(i, j, k) < 1 or max(i, j, k) > nx - 2:
            continue
        want = np.zeros(n)
        want[r] = h * h * v.sum()
        want[r - 1] -= h * h * v[0]
        want[r - nx] -= h * h * v[1]
        want[r - nx * nx] -= h * h * v[2]
        assert np.abs(C[r] - want).max() <= 1e-13 * h * h * v.sum(), r
        checked += 1
    assert checked == (nx - 2) ** 3


def test_gpu_full_upwind_conserves_and_has_upwind_signs(ctx):
    """seeded 16-mode curl field (the 3D convection-diffusion problem on
    3^3 hexes refined twice): convective part C = A(v) - A(0) has zero
    column sums on columns none of whose rows is a Dirichlet row, C_ij <= 0
    for i != j and C_ii >= 0"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import fields, problems
    cfg = problems.config("c4", nref=2)
    p = problems.Problem(ctx, cfg)
    A0 = ug.GPUSparseMatrix(ctx)
    d0 = ug.DomainDiscretization(p.hier)
    d0.set_diffusion(cfg["diffusion"])
    d0.assemble_jacobian(A0)
    n = p.n
    C = _dense(p.A, n) - _dense(A0, n)
    bnd = p.hier.export()[2].astype(bool)
    s = np.abs(C).max()
    assert s > 0
    # columns that no Dirichlet row couples to (structural pattern: the
    # Dirichlet rows keep their pattern with zero values)
    rp, ci, _ = A0.export_csr()
    touched = np.zeros(n, bool)
    for r in np.flatnonzero(bnd):
        touched[ci[rp[r]:rp[r + 1]]] = True
    cols = ~touched
    assert cols.sum() > 0
    assert np.abs(C[:, cols].sum(axis=0)).max() <= 1e-13 * s
    inner = ~bnd
    Ci = C[inner]
    off = Ci.copy()
    off[np.arange(inner.sum()), np.flatnonzero(inner)] = 0.0
    assert off.max() <= 1e-15 * s
    assert np.diag(C)[inner].min() >= -1e-15 * s
    assert fields.CurlField(cfg["vel_modes"], cfg["vel_kmax"], cfg["seed"] ^ fields.VEL_SEED_XOR).nmodes == 16
