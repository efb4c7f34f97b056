"""Generates the smoother fixtures in this folder from ugcore's OWN ILU(0)
and Gauss-Seidel smoothers.

Runs oracle/_ref/ref_smoothers (ug::ILU, ug::GaussSeidel,
ug::SymmetricGaussSeidel and ug::BackwardGaussSeidel compiled from the
reference sources by oracle/build_ref.sh) on the top-level operator of small
seeded oracle problems, with the multicolour ordering that the oracle's and
the GPU's smoothers use (rows ordered by (parity colour, index), the colour
(i & 1) | (j & 1) << 1 | (k & 1) << 2 of the structured grid vertex): ILU
gets it through ILU::set_ordering_algorithm, the Gauss-Seidel kinds run on
the permuted system.  Stores, per problem: its parameters, a checksum of the
operator, the ordering, seeded defects d and, per smoother and SOR factor,
ugcore's corrections c = B d.

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_smoother_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_smoothers")
sys.path.insert(0, ROOT)

# name: (elem, mx, my, mz, nref, seed, coef_kind, vel_kind, diffusion, peclet)
CASES = {
    "smoothers_quad_r4": ("quad", 2, 2, 1, 4, 1, 0, 0, 1.0, 10.0),
    "smoothers_hex_r2": ("hex", 2, 2, 2, 2, 1, 0, 0, 1.0, 10.0),
    "smoothers_tet_lognormal_r1": ("tet", 4, 4, 4, 1, 1, 1, 0, 1.0, 10.0),
    "smoothers_hex_convection_r1": ("hex", 3, 3, 3, 1, 1, 3, 1, 1e-2, 10.0),
}
# (key, ref_smoothers kind, oracle smoother kind, SOR factor / damping,
#  steps: 0 one application, k > 0 the smoother as a k-step base solver)
SMOOTHERS = [("ilu", 0, 3, 1.0, 0), ("gs_1.0", 1, 1, 1.0, 0), ("gs_1.3", 1, 1, 1.3, 0), ("sgs_1.0", 2, 2, 1.0, 0),
             ("sgs_1.3", 2, 2, 1.3, 0), ("sgs_0.7", 2, 2, 0.7, 0), ("bgs_1.0", 3, 4, 1.0, 0), ("bgs_0.8", 3, 4, 0.8, 0),
             ("jacobi_0.6", 4, 0, 0.6, 0), ("ls5_jacobi_0.6", 4, 0, 0.6, 5), ("ls2_gs_1.0", 1, 1, 1.0, 2),
             ("ls3_sgs_1.3", 2, 2, 1.3, 3), ("ls3_bgs_0.8", 3, 4, 0.8, 3), ("ls4_ilu", 0, 3, 1.0, 4)]


def oracle_problem(orc, case, smoother=3, relax=1.0, steps=1):
    elem, mx, my, mz, nref, seed, ck, vk, diffusion, peclet = case
    et = {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET}[elem]
    # the smoother as the base solver of a one-level cycle: one step from
    # zero gives c = B d, k steps the base solver's k corrections
    p = orc.make_params(elem_type=et, mx=mx, my=my, mz=mz, nref=nref, seed=seed, coef_kind=ck, vel_kind=vk,
                        diffusion=diffusion, peclet=peclet, smoother=smoother, damp=relax, base=nref,
                        base_steps=steps)
    return orc.Problem(p)


def ordering(case):
    """perm[i] = position of vertex i among the rows sorted by (colour, index)"""
    elem, mx, my, mz, nref = case[:5]
    nx, ny = mx * 2 ** nref + 1, my * 2 ** nref + 1
    nz = 1 if elem == "quad" else mz * 2 ** nref + 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    colour = ((i & 1) | ((j & 1) << 1) | ((k & 1) << 2)).ravel()
    order = np.lexsort((np.arange(colour.size), colour))
    perm = np.empty(colour.size, np.int64)
    perm[order] = np.arange(colour.size)
    return perm


def run(name, case):
    from oracle import oracle as orc
    orc.build()
    P = oracle_problem(orc, case)
    rp, ci, va = P.matrix()
    n = rp.size - 1
    perm = ordering(case)
    assert perm.size == n
    d = np.random.default_rng(17).standard_normal((3, n))
    out = {}
    for key, kind, _, relax, steps in SMOOTHERS:
        inp, res = "/tmp/smoothers_%s.in" % name, "/tmp/smoothers_%s.out" % name
        with open(inp, "wb") as f:
            np.asarray([n], np.int32).tofile(f)
            np.asarray([ci.size], np.int64).tofile(f)
            rp.astype(np.int32).tofile(f)
            ci.astype(np.int32).tofile(f)
            va.astype(np.float64).tofile(f)
            perm.tofile(f)
            np.asarray([kind], np.int32).tofile(f)
            np.asarray([relax], np.float64).tofile(f)
            np.asarray([steps], np.int32).tofile(f)
            np.asarray([d.shape[0]], np.int32).tofile(f)
            d.astype(np.float64).tofile(f)
        r = subprocess.run([DRIVER, inp, res], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(r.stderr)
        out["c_" + key] = np.fromfile(res, np.float64).reshape(d.shape)
    np.savez(os.path.join(HERE, name + ".npz"), elem=np.asarray(case[0]), params=np.asarray(case[1:], np.float64),
             nnz=ci.size, val_sum=float(np.abs(va).sum()), perm=perm, d=d, **out)
    print(name, n, "rows", ci.size, "entries")


if __name__ == "__main__":
    for nm, cs in CASES.items():
        run(nm, cs)
