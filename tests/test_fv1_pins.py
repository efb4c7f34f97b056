"""FV1 element values pinned outside the oracle's own restatement.

1. Against ugcore's code: tests/golden/fv1geom.npz holds what ugcore's own
   FV1Geometry (lib_disc/spatial_disc/disc_util/fv1_geom.cpp:259-464) and
   ConvectionShapesFullUpwind (conv_shape.h:277-345), compiled from the
   reference sources, compute for seeded distorted quadrilaterals,
   hexahedra, tetrahedra and triangles (tests/golden/make_fv1geom_golden.py).
   The oracle's geometry must reproduce SCV volumes, SCVF corners, area
   normals, integration points and shape gradients to 1e-13 relative, and
   its assembled diffusion operator on the fixture meshes the operator built
   from ugcore's geometry.
2. Independent of any FV1 code (mathematics only):
   (i)  on simplices the box-method diffusion operator with K constant per
        element equals the P1 finite-element stiffness sum_T K_T |T|
        grad(phi_i).grad(phi_j) (the SCVF normals of vertex i inside T sum
        to -|T| grad(phi_i)), on distorted meshes with lognormal K;
   (ii) on uniform grids the interior rows are the closed-form box stencils
        of bilinear / trilinear elements with SCVF integration points at the
        patch centres: quadrilaterals (any h) centre 3, axis neighbours -1/2,
        diagonal neighbours -1/4; hexahedra (spacing h) h * (27/8 centre,
        -3/16 axis, -5/32 face-diagonal, -3/64 corner neighbours).
Tolerance: 1e-13 relative to the row's largest entry (1e-13 of the element
scale for geometry).
"""
import os

import numpy as np
import pytest

from helpers import GOLDEN, oracle_params

FIX = os.path.join(GOLDEN, "fv1geom.npz")
TYPES = ["quad", "hex", "tet", "tri"]


@pytest.fixture(scope="module")
def fix():
    return dict(np.load(FIX))


def _orc_type(orc, t):
    return {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET, "tri": orc.ORC_TRI}[t]


@pytest.mark.parametrize("t", TYPES)
def test_oracle_geometry_matches_ugcore_fv1geometry(oracle_lib, fix, t):
    cs = fix["e_%s_corners" % t]
    for e in range(len(cs)):
        g = oracle_lib.geometry(_orc_type(oracle_lib, t), cs[e])
        size = np.ptp(cs[e], axis=0).max()
        dim = cs.shape[2]
        assert np.array_equal(g["frm"], fix["e_%s_frm" % t][e]) and np.array_equal(g["to"], fix["e_%s_to" % t][e])
        np.testing.assert_allclose(g["vols"], fix["e_%s_vol" % t][e], rtol=0, atol=1e-13 * size ** dim)
        np.testing.assert_allclose(g["normals"], fix["e_%s_normal" % t][e], rtol=0, atol=1e-13 * size ** (dim - 1))
        np.testing.assert_allclose(g["ips"], fix["e_%s_ip" % t][e], rtol=0, atol=1e-13 * size)
        np.testing.assert_allclose(g["grads"], fix["e_%s_grad" % t][e], rtol=0, atol=1e-13 / size)


def _boundary(coords):
    return np.any((coords == 0.0) | (coords == 1.0), axis=1).astype(np.uint8)


def _dense(rp, ci, va, n):
    A = np.zeros((n, n))
    A[np.repeat(np.arange(n), np.diff(rp)), ci] = va
    return A


def _assert_rows(A, R, bnd, rtol=1e-13):
    """non-Dirichlet rows of A equal R's (relative to R's row maximum);
    Dirichlet rows are identity rows"""
    inner = ~bnd.astype(bool)
    scale = np.abs(R[inner]).max(axis=1, keepdims=True)
    err = np.abs(A[inner] - R[inner]) / scale
    assert err.max() <= rtol, err.max()
    nb = np.flatnonzero(bnd)
    assert np.array_equal(A[nb], np.eye(A.shape[0])[nb])


def _oracle_mesh_matrix(orc, t, coords, elems, logk):
    from ugcore_gb300 import problems
    cfg = problems.config("c0", elem={"tri": "quad"}.get(t, t), coef="logk", nref=0)
    par = oracle_params(orc, cfg)
    par.elem_type = _orc_type(orc, t)
    par.nref = 0
    bnd = _boundary(coords)
    op = orc.Problem(par, m_top=logk, levels=[(np.ascontiguousarray(coords), np.ascontiguousarray(elems, np.int32),
                                               bnd, None, None)])
    rp, ci, va = op.matrix()
    return _dense(rp, ci, va, len(coords)), bnd


@pytest.mark.parametrize("t", TYPES)
def test_oracle_mesh_operator_matches_ugcore_geometry(oracle_lib, fix, t):
    coords, elems, logk = fix["m_%s_coords" % t], fix["m_%s_elems" % t], fix["m_%s_logK" % t]
    A, bnd = _oracle_mesh_matrix(oracle_lib, t, coords, elems, logk)
    _assert_rows(A, fix["m_%s_A_diffusion" % t], bnd)


def p1_stiffness(coords, elems, K):
    """P1 finite-element stiffness sum_T K_T |T| grad(phi_i).grad(phi_j)"""
    n, dim = coords.shape
    A = np.zeros((n, n))
    for e, el in enumerate(elems):
        X = coords[el]
        D = (X[1:] - X[0]).T                       # dim x dim
        vol = abs(np.linalg.det(D)) / (2.0 if dim == 2 else 6.0)
        G = np.linalg.solve(D.T, np.vstack([-np.ones(dim), np.eye(dim)]).T).T   # grads of phi, (dim+1) x dim
        A[np.ix_(el, el)] += K[e] * vol * (G @ G.T)
    return A


@pytest.mark.parametrize("t", ["tet", "tri"])
def test_box_method_equals_p1_fem_on_simplices(oracle_lib, fix, t):
    """(i) for the fixture meshes: ugcore's geometry operator, and the
    oracle's, equal the P1 stiffness"""
    coords, elems, logk = fix["m_%s_coords" % t], fix["m_%s_elems" % t], fix["m_%s_logK" % t]
    S = p1_stiffness(coords, elems, np.exp(logk))
    R = fix["m_%s_A_diffusion" % t]
    assert np.abs(R - S).max() <= 1e-13 * np.abs(S).max()
    A, bnd = _oracle_mesh_matrix(oracle_lib, t, coords, elems, logk)
    _assert_rows(A, S, bnd)


QUAD_STENCIL = {(0, 0): 3.0, (1, 0): -0.5, (-1, 0): -0.5, (0, 1): -0.5, (0, -1): -0.5,
                (1, 1): -0.25, (1, -1): -0.25, (-1, 1): -0.25, (-1, -1): -0.25}


def hex_stencil():
    st = {}
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                nz = abs(dx) + abs(dy) + abs(dz)
                st[(dx, dy, dz)] = {0: 27 / 8, 1: -3 / 16, 2: -5 / 32, 3: -3 / 64}[nz]
    return st


def check_box_stencil(rp, ci, va, nx, dim, h):
    """interior rows (all neighbours interior) against the closed form"""
    st = QUAD_STENCIL if dim == 2 else hex_stencil()
    scale = 1.0 if dim == 2 else h
    n = nx ** dim
    checked = 0
    for r in range(n):
        idx = [(r // nx ** d) % nx for d in range(dim)]
        if any(i < 2 or i > nx - 3 for i in idx):
            continue
        cols, vals = ci[rp[r]:rp[r + 1]], va[rp[r]:rp[r + 1]]
        want = {}
        for off, v in st.items():
            c = sum((idx[d] + off[d]) * nx ** d for d in range(dim))
            want[c] = v * scale
        assert sorted(want) == list(cols)
        got = dict(zip(cols.tolist(), vals.tolist()))
        for c, v in want.items():
            assert abs(got[c] - v) <= 1e-13 * 27 / 8 * scale, (r, c, got[c], v)
        checked += 1
    assert checked > 0
    return checked


@pytest.mark.parametrize("elem,nref", [("quad", 3), ("hex", 2)])
def test_oracle_uniform_grids_give_closed_form_box_stencils(oracle_lib, elem, nref):
    """(ii) K = 1 on the unit square / cube split into 2^d cells"""
    from ugcore_gb300 import problems
    cfg = problems.config("c0" if elem == "quad" else "c1", nref=nref)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg))
    rp, ci, va = op.matrix()
    nx = 2 * (1 << nref) + 1
    check_box_stencil(rp, ci, va, nx, 2 if elem == "quad" else 3, 1.0 / (nx - 1))


def test_fixture_stencils_are_consistent(fix):
    """the ugcore-geometry element matrices of the fixtures: rows and
    columns of the diffusion part sum to 0 (constants are in the kernel,
    fluxes are conservative), the convective part's column sums are 0 and
    its off-diagonals are <= 0 (full upwind)"""
    for t in ("hex", "tet"):
        A, D = fix["m_%s_A" % t], fix["m_%s_A_diffusion" % t]
        C = A - D
        s = np.abs(A).max()
        assert np.abs(D.sum(axis=1)).max() <= 1e-13 * s and np.abs(D.sum(axis=0)).max() <= 1e-13 * s
        assert np.abs(C.sum(axis=0)).max() <= 1e-13 * s
        off = C - np.diag(np.diag(C))
        assert off.max() <= 1e-15 * s and np.diag(C).min() >= -1e-15 * s
        assert np.abs(C).max() > 0.01 * s          # the convection is not negligible
