"""Matrix / vector files of device objects (SaveMatrixToMTX, ReadMatrixFromMTX,
SaveMatrixForConnectionViewer, SaveVectorForConnectionViewer, LoadVector):
byte-identical to the files ugcore's own writers made (golden/io/) and,
read back, bit-identical to what ugcore's readers returned."""
import os

import numpy as np
import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu

IO = os.path.join(GOLDEN, "io")


@pytest.fixture(scope="module")
def cases():
    return dict(np.load(os.path.join(IO, "cases.npz")))


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def _golden(name):
    with open(os.path.join(IO, name), "rb") as f:
        return f.read()


def _device_matrix(ctx, cases, name):
    import ugcore_gb300 as ug
    A = ug.GPUSparseMatrix(ctx)
    A.set_csr(cases[name + "_rowptr"], cases[name + "_col"], cases[name + "_val"],
              num_cols=int(cases[name + "_ncols"]))
    return A


@pytest.mark.parametrize("name", ["quad_r1", "hex_r1", "sym", "skew", "prolong", "special"])
def test_save_matrix_to_mtx(ctx, tmp_path, cases, name):
    from ugcore_gb300 import matrix_io
    out = str(tmp_path / (name + ".mtx"))
    matrix_io.SaveMatrixToMTX(out, _device_matrix(ctx, cases, name))
    assert open(out, "rb").read() == _golden(name + ".mtx")


@pytest.mark.parametrize("name", ["quad_r1", "sym", "skew", "dup_in", "sym_in"])
def test_read_matrix_from_mtx(ctx, cases, name):
    import ugcore_gb300 as ug
    from ugcore_gb300 import matrix_io
    A = matrix_io.ReadMatrixFromMTX(os.path.join(IO, name + ".mtx"), ug.GPUSparseMatrix(ctx))
    rp, ci, va = A.export_csr()
    assert A.num_cols() == int(cases[name + "_read_ncols"])
    assert np.array_equal(rp, cases[name + "_read_rowptr"])
    assert np.array_equal(ci, cases[name + "_read_col"])
    assert np.array_equal(_bits(va), _bits(cases[name + "_read_val"]))


@pytest.mark.parametrize("name,elem,m", [("quad_r1", "quad", (2, 2, 1)), ("hex_r1", "hex", (2, 2, 2))])
def test_connection_viewer_files_on_grid_positions(ctx, tmp_path, cases, name, elem, m):
    """positions come from the grid level (the same vertices the fixtures used)"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import matrix_io
    hier = ug.StructuredHierarchy(ctx, elem, m[0], m[1], m[2], 1)
    out = str(tmp_path / (name + ".mat"))
    matrix_io.SaveMatrixForConnectionViewer(hier, _device_matrix(ctx, cases, name), out)
    assert open(out, "rb").read() == _golden(name + ".mat")
    d = 2 if elem == "quad" else 3
    v = ug.GPUVector(ctx, hier.num_vertices()).copy_from(cases["vec%dd" % d])
    vout = str(tmp_path / "v.vec")
    matrix_io.SaveVectorForConnectionViewer(hier, v, vout)
    assert open(vout, "rb").read() == _golden("vec%dd.vec" % d)
    w = matrix_io.LoadVector(ug.GPUVector(ctx, hier.num_vertices()), os.path.join(IO, "vec%dd.vec" % d))
    assert np.array_equal(_bits(w.numpy()), _bits(cases["vec%dd_read" % d]))
    cmp = ug.GPUVector(ctx, hier.num_vertices()).copy_from(cases["vec%dd_cmp" % d])
    dout = str(tmp_path / "d.vec")
    matrix_io.SaveVectorDiffForConnectionViewer(hier, v, cmp, dout)
    assert open(dout, "rb").read() == _golden("vec%dd_diff.vec" % d)


def test_assembled_operator_round_trip(ctx, tmp_path):
    """the assembled FV1 operator of a 33^3 hex level (0.97M entries) written
    and read back: same pattern, values to the 13 digits the format keeps"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import matrix_io, problems
    p = problems.Problem(ctx, problems.config("c1", nref=4))
    out = str(tmp_path / "A.mtx")
    matrix_io.SaveMatrixToMTX(out, p.A)
    B = matrix_io.ReadMatrixFromMTX(out, ug.GPUSparseMatrix(ctx))
    rp, ci, va = p.A.export_csr()
    keep = va != 0.0
    brp, bci, bva = B.export_csr()
    assert np.array_equal(bci, ci[keep])
    assert np.allclose(bva, va[keep], rtol=1e-12, atol=0)
    # the operator's Dirichlet rows make it general; its nonzeros are all listed
    with open(out) as f:
        assert f.readline().split()[-1] == "general"
        f.readline()
        assert int(f.readline().split()[2]) == int(keep.sum())
