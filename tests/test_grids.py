"""Unstructured hierarchies from UGX coarse grids, built on the host
(ug4gb_io_ugx_level, no GPU): counts, nesting, orientation and the Dirichlet
subsets through the refinement (GlobalMultiGridRefiner semantics)."""
import os

import numpy as np
import pytest

from helpers import GOLDEN

GRIDS = os.path.join(GOLDEN, "grids")
# (file, dirichlet subsets, predicate of the Dirichlet vertices on every level)
CASES = [
    ("square_tris", "Dirichlet", lambda x: x[:, 0] == 0.0),
    ("square_tris", None, lambda x: np.any((x == 0.0) | (x == 1.0), axis=1)),
    ("square_quads", "Boundary", lambda x: np.any((x == 0.0) | (x == 1.0), axis=1)),
    ("cube_tets", "Bottom", lambda x: x[:, 2] == 0.0),
    ("cube_tets", None, lambda x: np.any((x == 0.0) | (x == 1.0), axis=1)),
    ("cube_hexes", "Boundary", lambda x: np.any((x == 0.0) | (x == 1.0), axis=1)),
    ("cube_tets", "Bottom, Other", lambda x: np.any((x == 0.0) | (x == 1.0), axis=1)),
]
NREF = 3


@pytest.fixture(scope="module")
def mio(built_lib):
    from ugcore_gb300 import matrix_io
    return matrix_io


def _measure(L):
    x, e = L["coords"], L["elems"]
    if e.shape[1] == 3:
        a, b, c = x[e[:, 0]], x[e[:, 1]], x[e[:, 2]]
        return 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))
    if e.shape[1] == 4 and x.shape[1] == 3:
        a, b, c, d = (x[e[:, j]] for j in range(4))
        return np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a)) / 6.0
    if e.shape[1] == 4:   # quadrilateral: shoelace
        s = 0.0
        for j in range(4):
            p, q = x[e[:, j]], x[e[:, (j + 1) % 4]]
            s = s + p[:, 0] * q[:, 1] - q[:, 0] * p[:, 1]
        return 0.5 * s
    # hexahedron: 6 tets of the Kuhn split about the 0-6 diagonal
    v = 0.0
    for t in ((0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)):
        a, b, c, d = (x[e[:, j]] for j in t)
        v = v + np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a)) / 6.0
    return v


def _facets(L):
    e = L["elems"]
    k = e.shape[1]
    dim = L["coords"].shape[1]
    if dim == 2:
        loc = [(j, (j + 1) % k) for j in range(k)]
    elif k == 4:
        loc = [(0, 2, 1), (1, 2, 3), (0, 3, 2), (0, 1, 3)]
    else:
        loc = [(0, 3, 2, 1), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]
    keys = np.sort(np.concatenate([e[:, list(f)] for f in loc]), axis=1)
    _, cnt = np.unique(keys, axis=0, return_counts=True)
    return cnt


@pytest.mark.parametrize("name,dirichlet,pred", CASES)
def test_hierarchy_properties(mio, name, dirichlet, pred):
    path = os.path.join(GRIDS, name + ".ugx")
    prev = None
    for l in range(NREF + 1):
        L = mio.ugx_level(path, NREF, l, dirichlet)
        x, e = L["coords"], L["elems"]
        dim = x.shape[1]
        m = _measure(L)
        assert np.all(m > 0.0), "element with non-positive orientation"
        assert abs(m.sum() - 1.0) < 1e-12, "total measure of the unit square / cube"
        # conforming: every facet in one or two elements
        cnt = _facets(L)
        assert cnt.max() <= 2
        # Dirichlet vertices: exactly the ones of the subsets' geometry
        assert np.array_equal(L["dirichlet"].astype(bool), pred(x)), (name, l)
        if prev is not None:
            assert len(e) == len(prev["elems"]) * (4 if dim == 2 else 8)
            nv0 = len(prev["coords"])
            # old vertices first, unchanged; new vertices at their parents' average
            assert np.array_equal(x[:nv0], prev["coords"])
            npar, par = L["npar"], L["par"]
            assert np.all(npar[:nv0] == 1) and np.array_equal(par[:nv0, 0], np.arange(nv0))
            for n in (2, 4, 8):
                sel = npar == n
                if sel.any():
                    avg = prev["coords"][par[sel, :n]].mean(axis=1)
                    assert np.allclose(x[sel], avg, rtol=0, atol=1e-15)
            assert set(np.unique(npar)) <= {1, 2, 4, 8}
        prev = L


def test_ugx_errors(mio, tmp_path):
    from ugcore_gb300 import UG4GBError
    path = os.path.join(GRIDS, "square_tris.ugx")
    with pytest.raises(UG4GBError, match="no subset named"):
        mio.ugx_level(path, 1, 1, "Nowhere")
    with pytest.raises(UG4GBError, match="cannot open"):
        mio.ugx_level(str(tmp_path / "missing.ugx"), 1, 0)
    bad = tmp_path / "prisms.ugx"
    bad.write_text('<grid><vertices coords="3">0 0 0 1 0 0 0 1 0 0 0 1 1 0 1 0 1 1</vertices>'
                   '<prisms>0 1 2 3 4 5</prisms></grid>')
    with pytest.raises(UG4GBError, match="not supported"):
        mio.ugx_level(str(bad), 0, 0)


@pytest.mark.parametrize("name,dirichlet", [("square_tris", "Dirichlet"), ("cube_tets", "Bottom"),
                                            ("cube_hexes", None)])
def test_oracle_solves_on_the_hierarchy(mio, oracle_lib, name, dirichlet):
    """the oracle's FV1 + GMG-PCG on the hierarchy levels converges (its
    triangle geometry included) and the operator has zero row sums away from
    the Dirichlet rows (constant K, no convection)"""
    path = os.path.join(GRIDS, name + ".ugx")
    nref = 2
    levels = []
    for l in range(nref + 1):
        L = mio.ugx_level(path, nref, l, dirichlet)
        levels.append((L["coords"], L["elems"], L["dirichlet"], L["npar"], L["par"]))
    et = {0: oracle_lib.ORC_QUAD, 1: oracle_lib.ORC_HEX, 2: oracle_lib.ORC_TET, 3: oracle_lib.ORC_TRI}[L["elem_type"]]
    op = oracle_lib.Problem(oracle_lib.make_params(elem_type=et, seed=2, rel_red=1e-10), levels=levels)
    rp, ci, va = op.matrix()
    rows = np.add.reduceat(va, rp[:-1])
    inner = ~L["dirichlet"].astype(bool)
    # an FV1 diffusion row (constant K) sums to zero: the flux of a constant vanishes
    assert np.abs(rows[inner]).max() < 1e-12 * np.abs(va).max()
    rs = op.solve()
    assert rs["steps"] < 40
    import scipy.sparse as sp
    A = sp.csr_matrix((va, ci, rp))
    r = A @ rs["x"] - op.rhs()
    assert np.linalg.norm(r) < 1e-9 * np.linalg.norm(op.rhs())


MALFORMED_UGX = [
    "",
    "<grid>",
    '<grid><vertices coords="3">0 0 0 1 0</vertices><tetrahedrons>0 1 2 3</tetrahedrons></grid>',
    '<grid><vertices coords="2">0 0 1 0 0 1</vertices><triangles>0 1 7</triangles></grid>',
    '<grid><vertices coords="2">0 0 1 0 0 1</vertices><triangles>0 1</triangles></grid>',
    '<grid><vertices coords="2">0 0 1 0 0 1</vertices><triangles>0 1 -3</triangles></grid>',
    '<grid><vertices coords="9">0 0 0</vertices></grid>',
    '<grid><vertices coords="2">0 0 1 0 0 1</vertices><triangles>0 1 2</triangles>'
    '<subset_handler name="defSH"><subset name="A"><vertices>0 5</vertices></subset></subset_handler></grid>',
    '<grid><vertices coords="2">0 0 1 0 0 1</vertices><triangles>0 1 2</triangles>'
    '<subset_handler name="defSH"><subset name="A"><edges>9</edges></subset></subset_handler></grid>',
    '<grid><vertices coords="2">a b c d e f</vertices><triangles>0 1 2</triangles></grid>',
]


@pytest.mark.parametrize("k", range(len(MALFORMED_UGX)))
def test_malformed_ugx_files_are_rejected(mio, tmp_path, k):
    """malformed UGX grids: an error with a message or a consistent level,
    never a crash (also run under the sanitizers, test_sanitizers.py)"""
    from ugcore_gb300 import UG4GBError
    f = tmp_path / ("g%d.ugx" % k)
    f.write_text(MALFORMED_UGX[k])
    try:
        L = mio.ugx_level(str(f), 1, 1, "A" if "subset" in MALFORMED_UGX[k] else None)
    except UG4GBError as e:
        assert str(e)
        return
    assert L["elems"].min() >= 0 and L["elems"].max() < len(L["coords"])
