"""Generates the golden fixtures in this folder from ugcore's OWN algebra.

Runs oracle/_ref/ref_driver (ugcore's SparseMatrix, SetDirichletRow,
set_as_transpose_of, Jacobi, LU, CG, BiCGStab and StdConvCheck compiled from
the reference sources by oracle/build_ref.sh) on small seeded problems and
stores, per case: every level's CRS, the top level's P and R, the rhs, the
solution, the defect history and the iteration count.

The *_rap cases build the coarse operators as Galerkin products with
ugcore's own AddMultiplyOf (the multigrid's set_rap(true) path).

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_golden.py [case ...]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name: (elem, mx, my, mz, nref, seed, coef_kind, solver, vel_kind, diffusion, peclet)
CASES = {
    "quad_2x2_r4": (0, 2, 2, 1, 4, 1, 0, 0, 0, 1.0, 10.0),
    "hex_2x2x2_r2": (1, 2, 2, 2, 2, 1, 0, 0, 0, 1.0, 10.0),
    "tet_4x4x4_r1_lognormal": (2, 4, 4, 4, 1, 1, 1, 0, 0, 1.0, 10.0),
    "hex_3x3x3_r1_convection": (1, 3, 3, 3, 1, 1, 3, 1, 1, 1e-2, 10.0),
}
# + (smoother, damp, nu1, nu2, maxit, rap)
RAP = (0, 0.6, 2, 2, 200, 1)
CASES.update({
    "hex_2x2x2_r2_rap": CASES["hex_2x2x2_r2"] + RAP,
    "tet_4x4x4_r1_lognormal_rap": CASES["tet_4x4x4_r1_lognormal"] + RAP,
    "hex_3x3x3_r1_convection_rap": CASES["hex_3x3x3_r1_convection"] + RAP,
})
# + (bicg_restart, bicg_min_ortho): BiCGStab::set_restart / set_min_orthogonality
NORAP = (0, 0.6, 2, 2, 200, 0)
CONV2 = (1, 3, 3, 3, 2, 1, 3, 1, 1, 1e-2, 10.0)
CASES.update({
    "hex_3x3x3_r2_convection_restart2": CONV2 + NORAP + (2, 0.0),
    "hex_3x3x3_r2_convection_minortho": CONV2 + NORAP + (0, 0.1),
    "hex_3x3x3_r2_convection_restart4_minortho": CONV2 + NORAP + (4, 0.3),
})
# + (damp_prol, damp_res): StdTransfer::set_prolongation_damping / set_restriction_damping
CASES.update({
    "hex_2x2x2_r2_damped": CASES["hex_2x2x2_r2"] + NORAP + (0, 0.0, 0.8, 1.25),
    "tet_4x4x4_r1_lognormal_damped": CASES["tet_4x4x4_r1_lognormal"] + NORAP + (0, 0.0, 1.3, 0.7),
})


def read_ref(path):
    buf = open(path, "rb").read()
    off = [0]

    def take(dt, n):
        a = np.frombuffer(buf, dt, n, off[0])
        off[0] += a.nbytes
        return a.copy()

    nl, steps, ok, nh = take(np.int32, 4)
    d0, d1, tset, tsol = take(np.float64, 4)

    def crs():
        n = int(take(np.int32, 1)[0])
        nnz = int(take(np.int64, 1)[0])
        return take(np.int32, n + 1), take(np.int32, nnz), take(np.float64, nnz)

    A = [crs() for _ in range(nl)]
    PR = [(crs(), crs()) for _ in range(nl - 1)]
    nv = len(A[-1][0]) - 1
    b = take(np.float64, nv)
    x = take(np.float64, nv)
    h = take(np.float64, nh)
    return dict(nl=int(nl), steps=int(steps), ok=int(ok), d0=d0, d1=d1, A=A, PR=PR, b=b, x=x, hist=h)


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build oracle/_ref first: sh oracle/build_ref.sh")
    names = sys.argv[1:] or list(CASES)
    for name in names:
        c = CASES[name]
        out = "/tmp/_golden_%s.bin" % name
        args = [DRIVER, out] + [str(v) if not isinstance(v, float) else repr(v) for v in c]
        subprocess.check_call(args, stdout=subprocess.DEVNULL)
        R = read_ref(out)
        os.remove(out)
        data = dict(params=np.array(c, dtype=np.float64), steps=R["steps"], ok=R["ok"], b=R["b"], x=R["x"],
                    hist=R["hist"], nlev=R["nl"])
        for l, (rp, ci, va) in enumerate(R["A"]):
            data["A%d_rowptr" % l], data["A%d_col" % l], data["A%d_val" % l] = rp, ci, va
        top = R["nl"] - 1
        (prp, pci, pva), (rrp, rci, rva) = R["PR"][top - 1]
        data.update(P_rowptr=prp, P_col=pci, P_val=pva, R_rowptr=rrp, R_col=rci, R_val=rva)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, "levels", R["nl"], "steps", R["steps"], "n", len(R["b"]))


if __name__ == "__main__":
    main()
