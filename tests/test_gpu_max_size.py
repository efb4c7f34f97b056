"""The largest structured problems the 32-bit indices allow, and a clean
refusal beyond them.

Row pointers, column indices and element corner lists are 32-bit, as in the
defragmented CRS the library exports; the operator of a 3D hexahedral grid
has (3n - 2)^3 entries for n^3 vertices, so 385^3 (1.53e9 entries,
57 million DoFs) is the largest cube in this family that fits and 513^3
(3.6e9 entries) does not.  At 385^3 the oracle is too slow for a
comparison: the solves are checked by the relative residual, computed here
in FP64 from the exported operator's action, and by the multigrid's
mesh-independent step count (within +-2 of the 129^3 problem's).  The
refusals beyond: an error with a message before any kernel indexes past
32 bits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _steps_129(ctx, precision):
    from ugcore_gb300 import problems
    p = problems.Problem(ctx, problems.config("c1", precision=precision))
    return p.solve()["steps"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_largest_hex_problem_solves(ctx, precision):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    ref_steps = _steps_129(ctx, precision)
    p = problems.Problem(ctx, problems.config("c1", mx=3, my=3, mz=3, nref=7, precision=precision))
    assert p.n == 385 ** 3
    st = p.solve()
    assert st["converged"] and abs(st["steps"] - ref_steps) <= 2, (st["steps"], ref_steps)
    r = ug.GPUVector(ctx, p.n)
    p.A.apply(r, p.x)                    # r = A x
    res = r.numpy() - p.b.numpy()
    # the fresh residual; the solver stops on the recursively updated one,
    # which follows it to rounding (a factor 2 allowed)
    assert np.linalg.norm(res) <= 2e-10 * np.linalg.norm(p.b.numpy())


@pytest.mark.parametrize("elem,mx,what", [("hex", 4, "nnz exceeds int32"),
                                          ("tet", 4, "too many element corners")])
def test_beyond_32bit_indices_is_refused(ctx, elem, mx, what):
    """513^3 vertices: the hexahedral operator would have 3.6e9 entries (the
    assembly refuses it), the Kuhn tetrahedra 3.2e9 element corners (the
    grid refuses them); an error with a message, no partial result"""
    import ugcore_gb300 as ug
    with pytest.raises(ug.UG4GBError) as e:
        h = ug.StructuredHierarchy(ctx, elem, mx, mx, mx, 7)
        d = ug.DomainDiscretization(h)
        d.set_diffusion(1.0)
        A = ug.GPUSparseMatrix(ctx)
        d.assemble_jacobian(A)
    assert what in str(e.value)
    ctx.synchronize()
