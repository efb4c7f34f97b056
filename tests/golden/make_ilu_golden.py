"""Generates the ILU fixtures in this folder from ugcore's OWN ILU(0).

Runs oracle/_ref/ref_ilu (ug::ILU<CPUAlgebra> compiled from the reference
sources by oracle/build_ref.sh) on the top-level operator of small seeded
oracle problems, with the multicolour ordering that the oracle's and the
GPU's ILU smoothers use (rows ordered by (parity colour, index), the colour
(i & 1) | (j & 1) << 1 | (k & 1) << 2 of the structured grid vertex) handed
to ILU::set_ordering_algorithm.  Stores, per case: the problem parameters, a
checksum of the operator, the ordering, seeded defects d and ugcore's
corrections c = (LU)^{-1} d.

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_ilu_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_ilu")
sys.path.insert(0, ROOT)

# name: (elem, mx, my, mz, nref, seed, coef_kind, vel_kind, diffusion, peclet)
CASES = {
    "ilu_quad_r4": ("quad", 2, 2, 1, 4, 1, 0, 0, 1.0, 10.0),
    "ilu_hex_r2": ("hex", 2, 2, 2, 2, 1, 0, 0, 1.0, 10.0),
    "ilu_tet_lognormal_r1": ("tet", 4, 4, 4, 1, 1, 1, 0, 1.0, 10.0),
    "ilu_hex_convection_r1": ("hex", 3, 3, 3, 1, 1, 3, 1, 1e-2, 10.0),
}


def oracle_problem(orc, case):
    elem, mx, my, mz, nref, seed, ck, vk, diffusion, peclet = case
    et = {"quad": orc.ORC_QUAD, "hex": orc.ORC_HEX, "tet": orc.ORC_TET}[elem]
    # ILU (smoother kind 3) as the base solver of a one-level cycle: one step
    # from zero gives c = (LU)^{-1} d
    p = orc.make_params(elem_type=et, mx=mx, my=my, mz=mz, nref=nref, seed=seed, coef_kind=ck, vel_kind=vk,
                        diffusion=diffusion, peclet=peclet, smoother=3, damp=1.0, base=nref, base_steps=1)
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
    inp, out = "/tmp/ilu_%s.in" % name, "/tmp/ilu_%s.out" % name
    with open(inp, "wb") as f:
        np.asarray([n], np.int32).tofile(f)
        np.asarray([ci.size], np.int64).tofile(f)
        rp.astype(np.int32).tofile(f)
        ci.astype(np.int32).tofile(f)
        va.astype(np.float64).tofile(f)
        perm.tofile(f)
        np.asarray([d.shape[0]], np.int32).tofile(f)
        d.astype(np.float64).tofile(f)
    r = subprocess.run([DRIVER, inp, out], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    c = np.fromfile(out, np.float64).reshape(d.shape)
    np.savez(os.path.join(HERE, name + ".npz"), elem=np.asarray(case[0]), params=np.asarray(case[1:], np.float64),
             nnz=ci.size, val_sum=float(np.abs(va).sum()), perm=perm, d=d, c=c)
    print(name, n, "rows", ci.size, "entries")


if __name__ == "__main__":
    for nm, cs in CASES.items():
        run(nm, cs)
