"""Generates the Newton fixtures in this folder from ugcore's OWN NewtonSolver.

Runs oracle/_ref/ref_newton (ugcore's NewtonSolver, StandardLineSearch,
AssembledOperator, CG and StdConvCheck compiled from the reference sources by
oracle/build_ref.sh, over the oracle's assembly and multigrid) on small
seeded problems and stores, per case: Newton steps, return code, the accepted
lambda of every line search, the total number of linear steps, the solution
and the initial / final Newton defects.

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_newton_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_newton")

# name: (elem, mx, my, mz, nref, seed, coef_kind, diffusion, theta, dt, maxit, min_defect, reduction,
#        ls_max, ls_start, ls_reduce, ls_accept_best, ls_check_all, linear_reduction)
CASES = {
    "newton_quad_r4_ls": (0, 2, 2, 1, 4, 1, 0, 1.0, -1.0, 0.0, 10, 1e-50, 1e-10, 10, 2.0, 0.5, 0, 0, 1e-2),
    "newton_hex_r2_ls_accept_best": (1, 2, 2, 2, 2, 3, 0, 1.0, -1.0, 0.0, 10, 1e-50, 1e-10, 2, 4.0, 0.5, 1, 0, 1e-1),
    "newton_tet_lognormal_ls_check_all": (2, 2, 2, 2, 2, 5, 1, 1.0, -1.0, 0.0, 12, 1e-50, 1e-10, 4, 1.0, 0.5, 0, 1,
                                          1e-3),
    "newton_hex_theta_half": (1, 2, 2, 2, 2, 1, 0, 1.0, 0.5, 0.01, 10, 1e-50, 1e-10, 0, 1.0, 0.5, 0, 0, 1e-4),
    "newton_quad_plain": (0, 2, 2, 1, 4, 2, 0, 1.0, -1.0, 0.0, 10, 1e-50, 1e-10, 0, 1.0, 0.5, 0, 0, 1e-3),
}


def run(name, args):
    out = os.path.join("/tmp", "newton_%s.bin" % name)
    r = subprocess.run([DRIVER, out] + [repr(a) if isinstance(a, float) else str(a) for a in args],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    b = open(out, "rb").read()
    steps, rc, nv, nrec, lin = np.frombuffer(b[:20], np.int32)
    o = 20
    lam = np.frombuffer(b[o:o + 8 * nrec]).copy()
    o += 8 * nrec
    u = np.frombuffer(b[o:o + 8 * nv]).copy()
    o += 8 * nv
    d0, d1 = np.frombuffer(b[o:o + 16])
    return dict(args=np.array(args, dtype=np.float64), steps=steps, rc=rc, lambdas=lam, linear_steps=lin, u=u,
                d0=d0, d1=d1)


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        res = run(n, CASES[n])
        np.savez_compressed(os.path.join(HERE, n + ".npz"), **res)
        print(n, "steps", int(res["steps"]), "rc", int(res["rc"]), "lambdas", res["lambdas"].tolist(),
              "linear", int(res["linear_steps"]), "defect %.3e -> %.3e" % (res["d0"], res["d1"]))
