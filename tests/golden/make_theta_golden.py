"""Generates the theta-step fixtures in this folder from ugcore's OWN
ThetaTimeStep.

Runs oracle/_ref/ref_theta (ugcore's ThetaTimeStep and dense LU compiled from
the reference sources by oracle/build_ref.sh, over a domain discretisation
whose time-dependent assembly is the oracle's) and stores, per case and
step: the time scalings ugcore passed, the previous solution, the step's
operator values and right-hand side, the defect of a perturbed iterate and
the jacobian.

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_theta_golden.py
"""
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_theta")

# name: (elem, mx, my, mz, nref, seed, coef_kind, theta, dt, nsteps)
CASES = {
    "theta_quad_cn": (0, 2, 2, 1, 4, 1, 0, 0.5, 0.01, 3),
    "theta_hex_implicit_euler": (1, 2, 2, 2, 2, 3, 0, 1.0, 0.05, 3),
    "theta_tet_lognormal_explicit": (2, 2, 2, 2, 1, 5, 1, 0.0, 1e-3, 2),
    "theta_quad_lognormal_0.7": (0, 2, 2, 1, 3, 2, 1, 0.7, 0.02, 3),
}


def run(name, args):
    out = os.path.join("/tmp", "theta_%s.bin" % name)
    r = subprocess.run([DRIVER, out] + [repr(a) if isinstance(a, float) else str(a) for a in args],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    b = open(out, "rb").read()
    nv, nnz, ns = struct.unpack("3i", b[:12])
    o = 12
    rec = {k: [] for k in ("scales", "u_old", "A", "b", "d", "J")}
    for _ in range(ns):
        for k, n in (("scales", 4), ("u_old", nv), ("A", nnz), ("b", nv), ("d", nv), ("J", nnz)):
            rec[k].append(np.frombuffer(b[o:o + 8 * n]).copy())
            o += 8 * n
    res = {k: np.array(v) for k, v in rec.items()}
    res["args"] = np.array(args, dtype=np.float64)
    return res


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(CASES)):
        res = run(n, CASES[n])
        np.savez_compressed(os.path.join(HERE, n + ".npz"), **res)
        print(n, "steps", len(res["b"]), "scales", res["scales"][0].tolist())
