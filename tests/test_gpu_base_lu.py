"""The dense LU base solver: bases of at most 160 unknowns are factorised on
the device (one block, no host round trip in a re-initialisation), larger
ones on the host.  Both follow LUDecomp's partial pivoting (lib_algebra/
small_algebra/no_lapack/lu_decomp.h); the multigrid application must match
the oracle on either side of the limit, and a singular base matrix must be
reported on either path (by the initialisation on the host path, by the next
application or solve on the device path, whose factorisation is not waited
for).
"""
import numpy as np
import pytest

from helpers import oracle_params

pytestmark = pytest.mark.gpu

CASES = [
    ("c3", dict(nref=4, base=0)),            # 9 unknowns: device
    ("c3", dict(nref=4, base=1)),            # 25: device
    ("c3", dict(nref=4, base=2)),            # 81: device
    ("c1", dict(nref=2, mx=3, my=3, mz=3)),  # 64: device
    ("c1", dict(nref=2, mx=4, my=4, mz=4)),  # 125: device
    ("c4", dict(nref=2, precision="fp64")),  # 64, upwind convection: device
    ("c3", dict(nref=4, base=3)),            # 289: host
    ("c1", dict(nref=1, mx=5, my=5, mz=5)),  # 216: host
]


@pytest.mark.parametrize("name,over", CASES)
def test_gmg_apply_matches_oracle_on_both_paths(ctx, oracle_lib, name, over):
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    cfg = problems.config(name, **over)
    p = problems.Problem(ctx, cfg)
    op = oracle_lib.Problem(oracle_params(oracle_lib, cfg), m_top=getattr(p, "m_top", None))
    d = np.random.default_rng(3).standard_normal(p.n)
    _, _, bnd = p.hier.export()
    d[bnd.astype(bool)] = 0.0
    c_ref = op.apply_gmg(d)
    dv = ug.GPUVector(ctx, p.n).copy_from(d)
    cv = ug.GPUVector(ctx, p.n)
    p.gmg.apply(cv, dv)
    err = np.abs(cv.numpy() - c_ref).max() / np.abs(c_ref).max()
    assert err < 1e-12, err
    # a re-initialisation on new values refactorises (same results again)
    p.gmg.init(p.A)
    p.gmg.apply(cv, dv)
    assert np.abs(cv.numpy() - c_ref).max() / np.abs(c_ref).max() < 1e-12


@pytest.mark.parametrize("name,over,at_init", [("c0", dict(nref=3), False), ("c3", dict(nref=4, base=2), False),
                                               ("c3", dict(nref=4, base=3), True)])
def test_singular_base_is_reported(ctx, name, over, at_init):
    """zero diffusion: every interior row of the base operator vanishes.  The
    host factorisation (289 unknowns) reports it from the init; the device
    one (9 and 81 unknowns) from the next application, which waits anyway"""
    import ugcore_gb300 as ug
    from ugcore_gb300 import problems
    with pytest.raises(ug.UG4GBError) as ei:
        p = problems.Problem(ctx, problems.config(name, coef="const", diffusion=0.0, **over))
        p.gmg.init(p.A)
        assert not at_init, "the host factorisation reports from the init"
        cv, dv = ug.GPUVector(ctx, p.n), ug.GPUVector(ctx, p.n).copy_from(np.ones(p.n))
        p.gmg.apply(cv, dv)
    assert ei.value.code == -4
    if not at_init:
        # a solve with it reports the same
        with pytest.raises(ug.UG4GBError) as ei:
            p2 = problems.Problem(ctx, problems.config(name, coef="const", diffusion=0.0, **over))
            p2.solve()
        assert ei.value.code == -4
    # the context stays usable
    q = problems.Problem(ctx, problems.config("c0", nref=3))
    assert q.solve()["converged"]
