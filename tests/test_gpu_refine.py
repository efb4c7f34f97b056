"""Refinement of unstructured hierarchies on the device against the host
statement of the same rules (ug4gb_io_ugx_level): coordinates bit for bit,
elements, Dirichlet vertices and parents identical, on every level."""
import os
import re

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu

GRIDS = os.path.join(GOLDEN, "grids")
CASES = [
    ("square_tris", "Dirichlet", 4),
    ("square_tris", None, 3),
    ("square_quads", "Boundary", 4),
    ("cube_tets", "Bottom", 3),
    ("cube_tets", None, 3),
    ("cube_hexes", "Boundary", 3),
    ("cube_hexes", None, 2),
]


def _compare(ctx, path, dirichlet, nref):
    import ugcore_gb300 as ug
    from ugcore_gb300 import matrix_io
    hier = ug.UnstructuredHierarchy.from_ugx(ctx, path, nref, dirichlet)
    assert hier.num_levels == nref + 1
    for level in range(nref + 1):
        ref = matrix_io.ugx_level(path, nref, level, dirichlet)
        coords, elems, bnd = hier.export(level)
        assert coords.shape == ref["coords"].shape and elems.shape == ref["elems"].shape
        assert np.array_equal(coords.view(np.int64), ref["coords"].view(np.int64)), level
        assert np.array_equal(elems, ref["elems"]), level
        assert np.array_equal(bnd, ref["dirichlet"]), level
        if level:
            npar, par = hier.parents(level)
            assert np.array_equal(npar, ref["npar"]) and np.array_equal(par, ref["par"]), level


@pytest.mark.parametrize("name,dirichlet,nref", CASES)
def test_device_refinement_matches_host(ctx, name, dirichlet, nref):
    _compare(ctx, os.path.join(GRIDS, name + ".ugx"), dirichlet, nref)


@pytest.mark.parametrize("name,dirichlet", [("square_tris", "Dirichlet"), ("cube_tets", "Bottom"),
                                            ("cube_hexes", "Boundary")])
def test_device_refinement_of_perturbed_grids(tmp_path, ctx, name, dirichlet):
    """coordinates moved off the dyadic lattice (every average rounds, the
    octahedron cuts depend on rounded lengths)"""
    text = open(os.path.join(GRIDS, name + ".ugx")).read()
    m = re.search(r'(<vertices coords="(\d)">)([^<]*)(</vertices>)', text)
    x = np.array(m.group(3).split(), float)
    rng = np.random.default_rng(11)
    x = x + rng.uniform(-0.04, 0.04, x.shape) * (1.0 + 1e-3 * np.pi)
    body = " ".join(repr(float(v)) for v in x)
    path = str(tmp_path / (name + "_perturbed.ugx"))
    with open(path, "w") as f:
        f.write(text[:m.start(3)] + body + text[m.end(3):])
    _compare(ctx, path, dirichlet, 3)
