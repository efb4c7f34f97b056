"""MatrixMarket and ConnectionViewer files: the library's writers against the
files ugcore's own writers produced (golden/io/, made by
golden/make_io_golden.py with oracle/_ref/ref_io), byte for byte; its readers
against what ugcore's readers returned for those files, bit for bit.

These use the host-array entry points (ug4gb_io_*), which need no GPU."""
import os

import numpy as np
import pytest

from helpers import GOLDEN

IO = os.path.join(GOLDEN, "io")
MATRICES = ["quad_r1", "hex_r1", "sym", "skew", "diag", "prolong", "special"]


@pytest.fixture(scope="module")
def cases(built_lib):
    return dict(np.load(os.path.join(IO, "cases.npz")))


@pytest.fixture(scope="module")
def mio(built_lib):
    from ugcore_gb300 import matrix_io
    return matrix_io


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.int64)


def _golden(name):
    with open(os.path.join(IO, name), "rb") as f:
        return f.read()


def _matrix(cases, name):
    return cases[name + "_rowptr"], cases[name + "_col"], cases[name + "_val"], int(cases[name + "_ncols"])


@pytest.mark.parametrize("name", MATRICES)
def test_mtx_write_matches_ugcore(tmp_path, cases, mio, name):
    rp, ci, va, nc = _matrix(cases, name)
    out = str(tmp_path / (name + ".mtx"))
    mio.write_mtx(out, rp, ci, va, num_cols=nc)
    assert open(out, "rb").read() == _golden(name + ".mtx")


@pytest.mark.parametrize("tag,comment", [("custom", "%a custom comment"), ("plain", "no percent sign"),
                                         ("empty", "")])
def test_mtx_comment_variants(tmp_path, cases, mio, tag, comment):
    rp, ci, va, nc = _matrix(cases, "quad_r1")
    out = str(tmp_path / "c.mtx")
    mio.write_mtx(out, rp, ci, va, num_cols=nc, comment=comment)
    assert open(out, "rb").read() == _golden("quad_r1_comment_%s.mtx" % tag)


@pytest.mark.parametrize("name", MATRICES + ["dup_in", "sym_in", "skew_in", "int_in"])
def test_mtx_read_matches_ugcore(cases, mio, name):
    rp, ci, va, nc = mio.read_mtx(os.path.join(IO, name + ".mtx"))
    assert nc == int(cases[name + "_read_ncols"])
    assert np.array_equal(rp, cases[name + "_read_rowptr"])
    assert np.array_equal(ci, cases[name + "_read_col"])
    assert np.array_equal(_bits(va), _bits(cases[name + "_read_val"]))


@pytest.mark.parametrize("name,dim", [("quad_r1", 2), ("hex_r1", 3)])
def test_connection_viewer_matrix_matches_ugcore(tmp_path, cases, mio, name, dim):
    rp, ci, va, _ = _matrix(cases, name)
    out = str(tmp_path / (name + ".mat"))
    mio.write_cv_matrix(out, rp, ci, va, cases["pos%d" % dim])
    assert open(out, "rb").read() == _golden(name + ".mat")


@pytest.mark.parametrize("dim", [2, 3])
def test_connection_viewer_vector_matches_ugcore(tmp_path, cases, mio, dim):
    v = cases["vec%dd" % dim]
    out = str(tmp_path / "v.vec")
    mio.write_cv_vector(out, v, cases["pos%d" % dim])
    assert open(out, "rb").read() == _golden("vec%dd.vec" % dim)
    back = mio.read_cv_vector(os.path.join(IO, "vec%dd.vec" % dim), len(v))
    assert np.array_equal(_bits(back), _bits(cases["vec%dd_read" % dim]))


@pytest.mark.parametrize("dim", [2, 3])
def test_connection_viewer_vector_difference_matches_ugcore(tmp_path, cases, mio, dim):
    """WriteVector with a compare vector writes v - w (SaveVectorDiffForConnectionViewer)"""
    out = str(tmp_path / "d.vec")
    mio.write_cv_vector(out, cases["vec%dd" % dim] - cases["vec%dd_cmp" % dim], cases["pos%d" % dim])
    assert open(out, "rb").read() == _golden("vec%dd_diff.vec" % dim)


def test_round_trip_of_a_large_random_matrix(tmp_path, mio):
    """general matrix with 200k entries: write, read back, same CRS up to the
    13 significant digits the format keeps; zero values are dropped"""
    rng = np.random.default_rng(3)
    n, per = 20000, 10
    ci = np.sort(np.stack([rng.choice(n, per, replace=False) for _ in range(n)]), axis=1).astype(np.int32).ravel()
    rp = np.arange(0, n * per + 1, per, dtype=np.int32)
    va = rng.standard_normal(n * per) * 10.0 ** rng.integers(-20, 20, n * per)
    va[::97] = 0.0
    out = str(tmp_path / "big.mtx")
    mio.write_mtx(out, rp, ci, va)
    brp, bci, bva, nc = mio.read_mtx(out)
    keep = va != 0.0
    assert nc == n and len(bci) == keep.sum()
    rows = np.repeat(np.arange(n), per)[keep]
    assert np.array_equal(np.diff(brp), np.bincount(rows, minlength=n))
    assert np.array_equal(bci, ci[keep])
    assert np.allclose(bva, va[keep], rtol=1e-12, atol=0)


def test_errors_are_reported(tmp_path, mio):
    from ugcore_gb300 import UG4GBError
    rp = np.array([0, 1], np.int32)
    ci = np.array([0], np.int32)
    va = np.array([1.0])
    with pytest.raises(UG4GBError, match="mtx"):
        mio.write_mtx(str(tmp_path / "a.txt"), rp, ci, va)
    with pytest.raises(UG4GBError, match="could not be found"):
        mio.read_mtx(str(tmp_path / "missing.mtx"))
    bad = tmp_path / "dense.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(UG4GBError, match="sparse"):
        mio.read_mtx(str(bad))
    short = tmp_path / "short.mtx"
    short.write_text("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n2 2\n")
    with pytest.raises(UG4GBError, match="three values"):
        mio.read_mtx(str(short))
    out = tmp_path / "out.mtx"
    out.write_text("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n")
    with pytest.raises(UG4GBError, match="outside"):
        mio.read_mtx(str(out))
    unsorted = (np.array([0, 2], np.int32), np.array([1, 0], np.int32), np.array([1.0, 2.0]))
    with pytest.raises(UG4GBError, match="increasing"):
        mio.write_mtx(str(tmp_path / "u.mtx"), *unsorted, num_cols=2)
    with pytest.raises(UG4GBError, match="mat"):
        mio.write_cv_matrix(str(tmp_path / "m.mtx"), rp, ci, va, np.zeros((1, 2)))
    with pytest.raises(UG4GBError, match="entries"):
        mio.read_cv_vector(os.path.join(IO, "vec2d.vec"), 7)


MALFORMED_MTX = [
    "",                                                                   # empty file
    "%%MatrixMarket matrix coordinate real general\n",                   # no size line
    "%%MatrixMarket matrix coordinate real general\n3\n",                # short size line
    "%%MatrixMarket matrix coordinate real general\n-2 2 1\n1 1 1.0\n",  # negative size
    "%%MatrixMarket matrix coordinate real general\n2 2 5\n1 1 1.0\n",   # fewer entries than announced
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1.0\n",   # index 0
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 x 1.0\n",   # non-numeric index
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 nanx\n",  # bad value
    "%%MatrixMarket matrix coordinate real general\n99999999999 2 1\n1 1 1.0\n",   # size beyond int
    "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1.0 0.0\n",     # complex
    "%%MatrixMarket matrix coordinate real general\n2 2 1\n" + "1 " * 5000 + "\n",  # a very long line
    "%%MatrixMarket matrix coordinate real symmetric\n2 3 1\n1 1 1.0\n",  # non-square symmetric
]


@pytest.mark.parametrize("k", range(len(MALFORMED_MTX)))
def test_malformed_mtx_files_are_rejected_or_read_safely(tmp_path, mio, k):
    """malformed MatrixMarket files: an error with a message, or (for what
    the format allows) a consistent matrix; never a crash (this test also runs
    under AddressSanitizer/UndefinedBehaviorSanitizer in test_sanitizers.py)"""
    from ugcore_gb300 import UG4GBError
    f = tmp_path / ("m%d.mtx" % k)
    f.write_text(MALFORMED_MTX[k])
    try:
        rp, ci, va, nc = mio.read_mtx(str(f))
    except UG4GBError as e:
        assert str(e)
        return
    assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and len(ci) == rp[-1] == len(va)
    assert len(ci) == 0 or (ci.min() >= 0 and ci.max() < nc)


MALFORMED_VEC = ["", "1\n", "2\n0 0 1.0\n", "1\n0 0\n", "3\n0 0 1.0\n0 1 2.0\n", "1\nx y z\n"]


@pytest.mark.parametrize("k", range(len(MALFORMED_VEC)))
def test_malformed_cv_vectors_are_rejected_or_read_safely(tmp_path, mio, k):
    from ugcore_gb300 import UG4GBError
    f = tmp_path / ("v%d.vec" % k)
    f.write_text(MALFORMED_VEC[k])
    try:
        v = mio.read_cv_vector(str(f), 2)
        assert len(v) == 2
    except UG4GBError as e:
        assert str(e)
