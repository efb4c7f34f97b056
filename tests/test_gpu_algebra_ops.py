"""The rest of the SparseMatrix / Vector interface (set-up and glue
operations ugcore's algebra templates call) against numpy on the same data."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr(n=50, seed=0, empty_row=7):
    rng = np.random.default_rng(seed)
    rows = []
    for r in range(n):
        if r == empty_row:
            rows.append([])
            continue
        cols = sorted(set(rng.choice(n, 5, replace=False).tolist()) | {r})
        rows.append(cols)
    rp = np.cumsum([0] + [len(c) for c in rows]).astype(np.int32)
    ci = np.array([c for cs in rows for c in cs], np.int32)
    va = rng.standard_normal(len(ci))
    return rp, ci, va


def _dense(rp, ci, va, n):
    D = np.zeros((n, n))
    for r in range(n):
        D[r, ci[rp[r]:rp[r + 1]]] = va[rp[r]:rp[r + 1]]
    return D


def test_matrix_copy_scale_clear(ctx):
    import ugcore_gb300 as ug
    rp, ci, va = _csr()
    B = ug.GPUSparseMatrix(ctx).set_csr(rp, ci, va)
    A = ug.GPUSparseMatrix(ctx).set_as_copy_of(B, 2.0)
    rpa, cia, vaa = A.export_csr()
    assert np.array_equal(rpa, rp) and np.array_equal(cia, ci) and np.array_equal(vaa, 2.0 * va)
    A.scale(0.25)
    assert np.array_equal(A.export_csr()[2], 0.5 * va)
    A.clear_retain_structure()
    rpa, cia, vaa = A.export_csr()
    assert np.array_equal(cia, ci) and not vaa.any()
    A.resize_and_clear(6, 9)
    assert A.info() == (6, 9, 0)
    assert not A.export_csr()[0].any()


def test_apply_ignore_zero_rows_and_rows(ctx):
    import ugcore_gb300 as ug
    n = 50
    rp, ci, va = _csr(n)
    A = ug.GPUSparseMatrix(ctx).set_csr(rp, ci, va)
    w = np.random.default_rng(1).standard_normal(n)
    d0 = np.full(n, 3.5)
    dest = ug.GPUVector(ctx, n).copy_from(d0)
    A.apply_ignore_zero_rows(dest, -2.0, ug.GPUVector(ctx, n).copy_from(w))
    ref = -2.0 * (_dense(rp, ci, va, n) @ w)
    got = dest.numpy()
    assert got[7] == 3.5                                   # the row without entries keeps dest
    mask = np.arange(n) != 7
    assert np.abs(got[mask] - ref[mask]).max() <= 1e-14 * np.abs(ref).max()
    for r in (0, 7, 31):
        c, v = A.row(r)
        assert np.array_equal(c, ci[rp[r]:rp[r + 1]]) and np.array_equal(v, va[rp[r]:rp[r + 1]])


def test_add_entries(ctx):
    import ugcore_gb300 as ug
    n = 50
    rp, ci, va = _csr(n)
    A = ug.GPUSparseMatrix(ctx).set_csr(rp, ci, va)
    r = [0, 0, 3, 3]
    c = [0, 0, 3, int(ci[rp[3] + 1])]
    v = [1.0, 2.0, 0.5, -1.0]
    A.add_entries(r, c, v)
    D = _dense(*A.export_csr(), n)
    R = _dense(rp, ci, va, n)
    for rr, cc, vv in zip(r, c, v):
        R[rr, cc] += vv
    assert np.abs(D - R).max() <= 1e-14
    with pytest.raises(ug.UG4GBError, match="pattern"):
        A.add_entries([7], [7], [1.0])                      # row 7 has no entries


def test_vector_maxnorm_and_values(ctx):
    import ugcore_gb300 as ug
    x = np.random.default_rng(3).standard_normal(100001)
    x[55555] = -17.25
    v = ug.GPUVector(ctx, len(x)).copy_from(x)
    assert v.maxnorm() == 17.25
    idx = [0, 5, 100000, 55555]
    assert np.array_equal(v.get_values(idx), x[idx])
    v.set_values([1, 2], [9.0, -9.0])
    assert np.array_equal(v.get_values([1, 2]), [9.0, -9.0])
    with pytest.raises(ug.UG4GBError, match="range"):
        v.get_values([100001])
    assert ug.GPUVector(ctx, 0).maxnorm() == 0.0
