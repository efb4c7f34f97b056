"""Two damped-Jacobi steps per pass over the level operator (k_sweep2.cu)
against the one-step-per-launch kernels.

The fused smoother must give bit-identical multigrid corrections (same
row arithmetic, explicitly rounded, in the same diagonal order); inside a
Krylov solve only the summation order of the fused (z, r) product differs, so
the solves take the same number of steps and agree to rounding.  Cases cover
15- and 27-diagonal operators (Kuhn tets, hexes, upwind convection), level
sizes that leave ragged 32 x 8 tiles, and chunk heights that give odd numbers
of z chunks.  The fused smoother runs on FP32 (mixed-precision) levels only.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALL_LEVELS = 1 | 2              # fused smoother on FP32 levels of every size

CASES = [
    ("c1", dict(nref=3)),                                   # 27 diagonals, 17^3
    ("c1", dict(nref=2, mx=5, my=3, mz=7)),                 # ragged 21 x 13 x 29
    ("c2", dict(nref=3)),                                   # 15 diagonals (Kuhn tets), 33^3
    ("c2", dict(nref=2, mx=7, my=5, mz=3)),                 # ragged 29 x 21 x 13
    ("c4", dict(nref=3)),                                   # upwind convection, 25^3
]


def _problem(ctx, name, over, prec):
    from ugcore_gb300 import problems
    cfg = problems.config(name, precision=prec, **over)
    return problems.Problem(ctx, cfg)


def _ctx(mask, planes=None):
    import ugcore_gb300 as ug
    c = ug.Context(0)
    c.set_tuning(sweep_fusion=mask, sweep_planes=planes)
    return c


def _fused_launches(ctx, fn):
    ctx.profile_begin()
    fn()
    prof = ctx.profile_end()
    return sum(v[0] for k, v in prof.items() if "k_sweep2" in k)


@pytest.mark.parametrize("prec", ["mixed"])
@pytest.mark.parametrize("name,over", CASES)
def test_gmg_application_bit_identical(name, over, prec):
    import ugcore_gb300 as ug
    ref_ctx = _ctx(0)
    pr = _problem(ref_ctx, name, over, prec)
    rng = np.random.default_rng(7)
    d = rng.uniform(-1.0, 1.0, pr.n)
    dr = ug.GPUVector(ref_ctx, pr.n).copy_from(d)
    cr = ug.GPUVector(ref_ctx, pr.n)
    pr.gmg.apply(cr, dr)
    want = cr.numpy()
    assert _fused_launches(ref_ctx, lambda: pr.gmg.apply(cr, dr)) == 0
    for mask, planes in [(ALL_LEVELS, 16), (ALL_LEVELS, 3), (ALL_LEVELS, 2), (ALL_LEVELS, 128)]:
        ctx = _ctx(mask, planes)
        p = _problem(ctx, name, over, prec)
        dv = ug.GPUVector(ctx, p.n).copy_from(d)
        cv = ug.GPUVector(ctx, p.n)
        p.gmg.apply(cv, dv)
        got = cv.numpy()
        assert np.array_equal(got, want), (mask, planes, float(np.abs(got - want).max()))
        assert _fused_launches(ctx, lambda: p.gmg.apply(cv, dv)) > 0
        # a second application on the same objects (graph replay) gives the same
        p.gmg.apply(cv, dv)
        assert np.array_equal(cv.numpy(), want)


def test_fp64_levels_are_not_fused():
    """FP64 levels keep the one-step kernels (their steps are bound by the
    FP64 FMA rate, not by operator bytes)"""
    import ugcore_gb300 as ug
    p = _problem(_ctx(ALL_LEVELS), "c1", dict(nref=3), "fp64")
    c = ug.GPUVector(p.ctx, p.n)
    assert _fused_launches(p.ctx, lambda: p.gmg.apply(c, p.b)) == 0


@pytest.mark.parametrize("prec", ["mixed"])
@pytest.mark.parametrize("name,over", [("c1", dict(nref=4)), ("c2", dict(nref=3)), ("c4", dict(nref=3))])
def test_solve_agrees(name, over, prec):
    pr = _problem(_ctx(0), name, over, prec)
    p = _problem(_ctx(ALL_LEVELS), name, over, prec)
    s1, s2 = pr.solve(), p.solve()
    assert abs(s1["steps"] - s2["steps"]) <= 1
    assert s2["defect"] / s2["initial_defect"] < 1e-10
    x1, x2 = pr.x.numpy(), p.x.numpy()
    assert np.abs(x1 - x2).max() <= 1e-8 * np.abs(x1).max()


def test_wrapped_entries_keep_the_one_step_kernels():
    """a top-level operator with a nonzero entry towards a vertex outside the
    level (here: x = nx-1 coupled to x = 0 of the next grid line, offset +1)
    is not fused on that level; the lower levels still are, and the result
    stays identical to the unfused multigrid"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config("c1", nref=3, precision="mixed")
    out = []
    for mask in (0, ALL_LEVELS):
        ctx = _ctx(mask)
        p = problems.Problem(ctx, cfg)
        rp, ci, va = p.A.export_csr()
        nx = round(p.n ** (1.0 / 3.0))
        row = nx - 1 + nx * (nx // 2 + nx * (nx // 2))          # x = nx-1 on an interior line
        assert row + 1 not in ci[rp[row]:rp[row + 1]]
        cols = np.insert(ci[rp[row]:rp[row + 1]], np.searchsorted(ci[rp[row]:rp[row + 1]], row + 1), row + 1)
        vals = np.insert(va[rp[row]:rp[row + 1]], np.searchsorted(ci[rp[row]:rp[row + 1]], row + 1), -1e-3)
        ci2 = np.concatenate([ci[:rp[row]], cols, ci[rp[row + 1]:]]).astype(np.int32)
        va2 = np.concatenate([va[:rp[row]], vals, va[rp[row + 1]:]])
        rp2 = rp.copy()
        rp2[row + 1:] += 1
        A = ug.GPUSparseMatrix(ctx)
        A.set_csr(rp2, ci2, va2)
        g = p._make_gmg(transposed=False)
        g.init(A)
        d = ug.GPUVector(ctx, p.n).copy_from(np.random.default_rng(3).uniform(-1, 1, p.n))
        c = ug.GPUVector(ctx, p.n)
        g.apply(c, d)
        out.append(c.numpy())
        ctx.profile_begin()
        g.apply(c, d)
        prof = ctx.profile_end()
        top = "L%d|" % (p.hier.num_levels - 1)
        assert not any(k.startswith(top) and "k_sweep2" in k for k in prof)
        if mask:
            assert any("k_sweep2" in k for k in prof)
    assert np.array_equal(out[0], out[1])


def test_bounded_wait_gives_up_and_the_context_recovers():
    """failure detection without a fault: with the test-only setting
    UG4GB_TUNE_SWEEP_WAIT_TEST block 0 of the next fused sweep announces bytes
    that no copy delivers, so its bounded wait runs out (half a second); the
    block issues no further copies, still joins the grid reduction, and the
    solve reports UG4GB_ERR_CUDA.  The context stays usable: a solve on it
    afterwards (setting off, fresh multigrid) is bit-identical to a solve on
    a fresh context, so the error flag and the reduction counters were left
    clean."""
    import ugcore_gb300 as ug
    from ugcore_gb300 import _lib
    c = _ctx(ALL_LEVELS)
    c.set_tuning(sweep_wait_test=64)
    p = _problem(c, "c1", dict(nref=3), "mixed")
    with pytest.raises(ug.UG4GBError) as ei:
        p.solve()
    assert ei.value.code == _lib.ERR_CUDA and "bounded wait" in str(ei.value)
    c.set_tuning(sweep_wait_test=0)
    q = _problem(c, "c1", dict(nref=3), "mixed")
    s1 = q.solve()
    r = _problem(_ctx(ALL_LEVELS), "c1", dict(nref=3), "mixed")
    s2 = r.solve()
    assert s1["converged"] and s1["steps"] == s2["steps"]
    assert np.array_equal(q.x.numpy(), r.x.numpy())


def test_default_runs_no_fused_sweeps():
    """the fused pairs are opt-in: a default context launches none (and keeps
    no padded operator copy)"""
    import ugcore_gb300 as ug
    p = _problem(ug.Context(0), "c1", dict(nref=4), "mixed")
    c = ug.GPUVector(p.ctx, p.n)
    d = ug.GPUVector(p.ctx, p.n).copy_from(np.ones(p.n))
    assert _fused_launches(p.ctx, lambda: p.gmg.apply(c, d)) == 0
