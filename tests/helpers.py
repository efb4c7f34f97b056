"""Shared helpers of the parity tests: map a problems.py configuration onto
the oracle's parameters, compare CRS matrices, read golden fixtures."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Tolerances stated by the benchmark spec for this path:
#   CRS row pointers / column indices: bit-exact
#   matrix values: 1e-13 relative in FP64 (relative to the largest |a_ij| of
#     the row, so that entries that cancel to ~0 are measured against the row)
#   solution: 1e-10 relative residual, iteration count within +-1
VAL_RTOL = 1e-13


SMOOTHERS = {"jacobi": 0, "mcgs": 1, "mcsgs": 2, "ilu": 3, "mcbgs": 4}


def oracle_params(orc, cfg):
    et = {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET}[cfg["elem"]]
    if cfg["coef"] == "const":
        ck = 0 if (cfg["diffusion"] == 1.0) else 3
    else:
        ck = {"lognormal": 1, "logk": 2}[cfg["coef"]]
    return orc.make_params(
        elem_type=et, mx=cfg["mx"], my=cfg["my"], mz=cfg["mz"], nref=cfg["nref"], seed=cfg["seed"], coef_kind=ck,
        coef_modes=cfg["coef_modes"], coef_kmax=cfg["coef_kmax"], vel_kind=1 if cfg["vel"] else 0,
        vel_modes=cfg["vel_modes"], vel_kmax=cfg["vel_kmax"], diffusion=cfg["diffusion"], peclet=cfg["peclet"],
        solver=0 if cfg["solver"] == "cg" else 1, smoother=SMOOTHERS[cfg["smoother"]],
        damp=cfg["damp"], nu1=cfg["nu1"], nu2=cfg["nu2"], cycle=cfg["cycle"], base=cfg["base"], maxit=cfg["maxit"],
        rel_red=cfg["rel_red"], min_defect=cfg["min_defect"], rap=int(cfg.get("rap", 0)),
        bicg_restart=int(cfg.get("bicg_restart", 0)), bicg_min_ortho=float(cfg.get("bicg_min_ortho", 0.0)),
        damp_prol=float(cfg.get("damp_prol", 1.0)), damp_res=float(cfg.get("damp_res", 1.0)),
        post_smoother=SMOOTHERS[cfg["post_smoother"]] if cfg.get("post_smoother") else -1,
        post_damp=float(cfg.get("post_damp", 1.0)),
        base_steps=int(cfg.get("base_steps", 0)) if cfg.get("base_solver", "lu") == "smoother" else 0)


def assert_crs_equal(a, b, rtol=VAL_RTOL, what="matrix"):
    """a, b = (rowptr, col, val); pattern bit-exact, values row-relative."""
    rpa, cia, vaa = a
    rpb, cib, vab = b
    assert np.array_equal(rpa, rpb), what + ": row pointers differ"
    assert np.array_equal(cia, cib), what + ": column indices differ"
    n = len(rpa) - 1
    rowmax = np.maximum.reduceat(np.abs(vab), rpb[:-1]) if len(vab) else np.zeros(n)
    scale = np.repeat(rowmax, np.diff(rpb))
    err = np.abs(vaa - vab)
    bad = err > rtol * np.maximum(scale, 1e-300)
    assert not bad.any(), "%s: %d values beyond %.0e (max rel %.3e)" % (
        what, int(bad.sum()), rtol, float((err / np.maximum(scale, 1e-300)).max()))


def rel_residual(p, x):
    """|b - A x| / |b| of a problems.Problem for a host solution x"""
    import ugcore_gb300 as ug
    r = ug.GPUVector(p.ctx, p.n)
    xv = ug.GPUVector(p.ctx, p.n).copy_from(x)
    p.A.axpy(r, 1.0, p.b, -1.0, xv)
    return r.norm() / p.b.norm()


def reference_tree():
    """location of the ugcore source tree, or None where it is absent (asked
    of oracle/build_ref.sh, the recipe that compiles it)"""
    import subprocess
    r = subprocess.run(["sh", os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "build_ref.sh"), "--where"],
                       capture_output=True, text=True)
    where = r.stdout.strip()
    return where if r.returncode == 0 and where else None


def load_golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    return dict(np.load(path)) if os.path.exists(path) else None
