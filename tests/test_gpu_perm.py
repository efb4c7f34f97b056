"""DoF permutations between the engine's numbering and an external one (the
ugcore-side glue's boundary): vectors and operators against numpy, the
permutation from vertex positions, the value-only refill after a
re-assembly, and a solve in the external numbering."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dense(A, n):
    rp, ci, va = A.export_csr()
    D = np.zeros((n, n))
    D[np.repeat(np.arange(n), np.diff(rp)), ci] = va
    return D


def test_permuted_vectors_and_operator(ctx):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c2", nref=2))
    n = p.n
    perm = np.random.default_rng(3).permutation(n).astype(np.int32)
    P = ug.DofPermutation(ctx, perm)
    x = np.random.default_rng(4).standard_normal(n)
    xe = ug.GPUVector(ctx, n).copy_from(x)
    xx = P.vector(xe, ug.GPUVector(ctx, n), to_external=True)
    assert np.array_equal(xx.numpy(), x[perm])
    back = P.vector(xx, ug.GPUVector(ctx, n), to_external=False)
    assert np.array_equal(back.numpy(), x)
    B = P.matrix(p.A, ug.GPUSparseMatrix(ctx), to_external=True)
    D, DB = _dense(p.A, n), _dense(B, n)
    assert np.array_equal(DB, D[np.ix_(perm, perm)])
    rp, ci, _ = B.export_csr()
    assert all(np.all(np.diff(ci[rp[i]:rp[i + 1]]) > 0) for i in range(n))
    # a re-assembly of the same pattern refills the values only
    p.disc.set_diffusion(3.0)
    p.disc.assemble_linear(p.A, p.b)
    P.matrix(p.A, B, to_external=True)
    assert np.array_equal(_dense(B, n), _dense(p.A, n)[np.ix_(perm, perm)])
    # and back
    A2 = P.matrix(B, ug.GPUSparseMatrix(ctx), to_external=False)
    assert np.array_equal(_dense(A2, n), _dense(p.A, n))


def test_permutation_from_positions_and_external_solve(ctx):
    """positions of the vertices in a shuffled order give back the shuffle;
    the operator and rhs moved to that numbering solve to the permuted
    solution (CG with the engine's multigrid applied through the
    permutation is what the glue does)"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c1", nref=3))
    coords, _, _ = p.hier.export()
    perm = np.random.default_rng(5).permutation(p.n).astype(np.int32)
    P = ug.DofPermutation(ctx, hier=p.hier, positions=coords[perm] + 1e-12, tol=1e-9)
    x = np.arange(p.n, dtype=np.float64)
    xx = P.vector(ug.GPUVector(ctx, p.n).copy_from(x), ug.GPUVector(ctx, p.n))
    assert np.array_equal(xx.numpy(), x[perm])
    st = p.solve()
    u = p.x.numpy()
    B = P.matrix(p.A, ug.GPUSparseMatrix(ctx))
    bx = P.vector(p.b, ug.GPUVector(ctx, p.n))
    ux = P.vector(p.x, ug.GPUVector(ctx, p.n))
    r = ug.GPUVector(ctx, p.n)
    B.axpy(r, 1.0, bx, -1.0, ux)
    assert r.norm() / bx.norm() < 1e-10 and st["converged"]
    assert np.array_equal(ux.numpy(), u[perm])
    with pytest.raises(ug.UG4GBError):
        ug.DofPermutation(ctx, np.zeros(p.n, np.int32))          # not a bijection
