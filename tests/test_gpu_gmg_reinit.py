"""Re-initialising a multigrid with a new operator on the same hierarchy (what
Newton, time stepping and the adjoint gradient do every step) keeps its
level buffers and transfers; the result must be bit-identical to a
multigrid built fresh for that operator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("c1", dict(nref=4), {}),
    ("c1", dict(nref=4, precision="mixed"), {}),
    ("c1", dict(nref=4, rap=1), {}),
    ("c1", dict(nref=4, smoother="mcsgs"), {}),
    ("c1", dict(nref=4, smoother="ilu"), {}),
    ("c2", dict(nref=3, precision="mixed"), {}),
    ("c2", dict(nref=3, precision="fp64"), dict(transposed=True)),
    ("c3", dict(nref=5), {}),
]


@pytest.mark.parametrize("name,over,extra", CASES)
def test_reinit_matches_fresh_multigrid(ctx, name, over, extra):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    p = problems.Problem(ctx, cfg)
    tr = extra.get("transposed", False)
    g1 = p._make_gmg(tr)
    g1.init(p.A)
    d = np.random.default_rng(2).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    c0 = ug.GPUVector(ctx, p.n)
    g1.apply(c0, ug.GPUVector(ctx, p.n).copy_from(d))
    # a different operator on the same hierarchy
    p.disc.set_diffusion(2.5)
    A2, b2 = ug.GPUSparseMatrix(ctx), ug.GPUVector(ctx, p.n)
    p.disc.assemble_linear(A2, b2)
    g1.init(A2)
    g2 = p._make_gmg(tr)
    g2.init(A2)
    out = []
    for g in (g1, g2):
        c = ug.GPUVector(ctx, p.n)
        g.apply(c, ug.GPUVector(ctx, p.n).copy_from(d))
        out.append(c.numpy())
    assert not np.array_equal(out[0], c0.numpy())
    assert np.array_equal(out[0].view(np.int64), out[1].view(np.int64))
