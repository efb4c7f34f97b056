"""Generates the matrix / vector file fixtures in golden/io/ with ugcore's OWN
writers and readers.

Runs oracle/_ref/ref_io (ugcore's MatrixIOMtx::write_from / read_into and
ConnectionViewer::WriteMatrix / WriteVector / ReadVector, compiled from the
reference sources by oracle/build_ref.sh) on small matrices and vectors and
stores what they wrote (.mtx, .mat, .vec text files) and what they read back
(io/cases.npz).  The matrices are the oracle's FV1 operators and transfers
plus hand-made symmetric, skew-symmetric, diagonal and special-value ones;
positions are the lexicographic vertices of the unit square / cube.

Usage (needs the reference tree, i.e. this container):
    sh oracle/build_ref.sh && python tests/golden/make_io_golden.py
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "io")
REF_IO = os.path.join(ROOT, "oracle", "_ref", "ref_io")
sys.path.insert(0, ROOT)


def grid_positions(n, dim):
    """lexicographic vertices of [0,1]^dim with n per direction"""
    t = np.arange(n) / (n - 1)
    if dim == 2:
        y, x = np.meshgrid(t, t, indexing="ij")
        return np.stack([x.ravel(), y.ravel()], 1)
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], 1)


def to_dense(rp, ci, va, ncols):
    n = len(rp) - 1
    D = np.zeros((n, ncols))
    for r in range(n):
        D[r, ci[rp[r]:rp[r + 1]]] = va[rp[r]:rp[r + 1]]
    return D


def from_pattern(rp, ci, D):
    """CRS with the given pattern and the values of D (stored zeros kept)"""
    va = np.array([D[r, ci[a]] for r in range(len(rp) - 1) for a in range(rp[r], rp[r + 1])])
    return rp.copy(), ci.copy(), va


def union_pattern(rp, ci, n):
    """pattern of A + A^T"""
    rows = [set() for _ in range(n)]
    for r in range(n):
        for a in range(rp[r], rp[r + 1]):
            rows[r].add(int(ci[a]))
            rows[int(ci[a])].add(r)
    nrp = np.zeros(n + 1, np.int32)
    nci = []
    for r in range(n):
        c = sorted(rows[r])
        nci += c
        nrp[r + 1] = nrp[r] + len(c)
    return nrp, np.array(nci, np.int32)


def write_csr(path, rp, ci, va, ncols):
    with open(path, "wb") as f:
        f.write(struct.pack("<iiq", len(rp) - 1, ncols, len(ci)))
        f.write(np.asarray(rp, np.int32).tobytes())
        f.write(np.asarray(ci, np.int32).tobytes())
        f.write(np.asarray(va, np.float64).tobytes())


def read_csr(path):
    b = open(path, "rb").read()
    rows, cols, nnz = struct.unpack("<iiq", b[:16])
    o = 16
    rp = np.frombuffer(b, np.int32, rows + 1, o)
    o += 4 * (rows + 1)
    ci = np.frombuffer(b, np.int32, nnz, o)
    o += 4 * nnz
    va = np.frombuffer(b, np.float64, nnz, o)
    return rp.copy(), ci.copy(), va.copy(), cols


def write_pos(path, pos):
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", pos.shape[0], pos.shape[1]))
        f.write(np.ascontiguousarray(pos, np.float64).tobytes())


def run(*args):
    r = subprocess.run([REF_IO] + list(args), capture_output=True, text=True)
    if r.returncode:
        sys.exit("ref_io %s failed (%d): %s" % (" ".join(args), r.returncode, r.stderr))


def matrices():
    from oracle import oracle as orc
    orc.build()
    q = orc.Problem(orc.make_params(elem_type=orc.ORC_QUAD, mx=2, my=2, nref=1, seed=1))
    h = orc.Problem(orc.make_params(elem_type=orc.ORC_HEX, mx=2, my=2, mz=2, nref=1, seed=1))
    rp, ci, va = q.matrix()
    n = len(rp) - 1
    M = {"quad_r1": (rp, ci, va, n), "hex_r1": h.matrix() + (125,)}
    # symmetric: (A + A^T) / 2 on the union pattern, one pair of stored zeros
    urp, uci = union_pattern(rp, ci, n)
    D = to_dense(rp, ci, va, n)
    S = 0.5 * (D + D.T)
    S[6, 7] = S[7, 6] = 0.0
    M["sym"] = from_pattern(urp, uci, S) + (n,)
    # skew-symmetric off the diagonal (diagonal entries kept)
    K = 0.5 * (D - D.T)
    K[np.diag_indices(n)] = np.arange(1, n + 1) * 0.25
    K[3, 8] = 2.5
    K[8, 3] = -2.5
    M["skew"] = from_pattern(urp, uci, K) + (n,)
    M["diag"] = (np.arange(6, dtype=np.int32), np.arange(5, dtype=np.int32), np.arange(1.0, 6.0), 5)
    P = q.transfer(1, 0)
    M["prolong"] = (P[0], P[1], P[2], int(P[1].max()) + 1)
    sp_rp = np.array([0, 3, 5, 8, 10], np.int32)
    sp_ci = np.array([0, 1, 3, 1, 2, 0, 2, 3, 0, 3], np.int32)
    sp_va = np.array([1e-300, -1e300, 5e-324, 0.1, 1.0 / 3.0, -2.0 / 3.0, 123456789.123, -0.0, 0.0, -7.25])
    M["special"] = (sp_rp, sp_ci, sp_va, 4)
    return M


# MatrixMarket inputs for the reader (comment lines, duplicates, upper-triangle
# entries of symmetric files, integers).  ugcore's reader stops with an
# exception on an empty line between the comments and the sizes
# (matrix_io_mtx.cpp:207-217 reads str.at(0) of it), so none has one.
READ_INPUTS = {
    "dup_in": ("%%MatrixMarket matrix coordinate real general\n% first comment\n%second\n"
               "3 4 6\n3 4 1.5\n1 1 2\n2 3 -4.25e-3\n1 1 7\n3 1 0\n2 3 1e+2\n"),
    "sym_in": ("%%MatrixMarket matrix coordinate real symmetric\n4 4 5\n1 1 4.0\n2 1 -1.0\n"
               "3 4 0.5\n4 4 2\n2 2 3.0\n"),
    "skew_in": "%%MatrixMarket matrix coordinate real skew-symmetric\n3 3 3\n2 1 1.25\n3 1 -2\n3 3 9\n",
    "int_in": "%%MatrixMarket matrix coordinate integer general\n2 2 3\n1 1 3\n2 1 -5\n2 2 12\n",
}


def main():
    if not os.path.exists(REF_IO):
        sys.exit("build oracle/_ref first: sh oracle/build_ref.sh")
    os.makedirs(OUT, exist_ok=True)
    store = {}
    pos = {2: grid_positions(5, 2), 3: grid_positions(5, 3)}
    with tempfile.TemporaryDirectory() as tmp:
        for d, p in pos.items():
            write_pos(os.path.join(tmp, "pos%d.bin" % d), p)
            store["pos%d" % d] = p
        for name, (rp, ci, va, ncols) in matrices().items():
            csr = os.path.join(tmp, name + ".csr")
            write_csr(csr, rp, ci, va, ncols)
            store[name + "_rowptr"], store[name + "_col"], store[name + "_val"] = rp, ci, va
            store[name + "_ncols"] = np.int64(ncols)
            mtx = os.path.join(OUT, name + ".mtx")
            if os.path.exists(mtx):
                os.remove(mtx)
            run("write-mtx", csr, mtx)
            back = os.path.join(tmp, name + "_back.csr")
            run("read-mtx", mtx, back)
            brp, bci, bva, bcols = read_csr(back)
            store[name + "_read_rowptr"], store[name + "_read_col"], store[name + "_read_val"] = brp, bci, bva
            store[name + "_read_ncols"] = np.int64(bcols)
            if name in ("quad_r1", "hex_r1"):
                d = 2 if name == "quad_r1" else 3
                run("write-mat", csr, os.path.join(tmp, "pos%d.bin" % d), os.path.join(OUT, name + ".mat"))
        # comment variants
        csr = os.path.join(tmp, "quad_r1.csr")
        for tag, comment in (("custom", "%a custom comment"), ("plain", "no percent sign"), ("empty", "")):
            mtx = os.path.join(OUT, "quad_r1_comment_%s.mtx" % tag)
            if os.path.exists(mtx):
                os.remove(mtx)
            run("write-mtx", csr, mtx, comment)
        # reader inputs
        for name, text in READ_INPUTS.items():
            src = os.path.join(OUT, name + ".mtx")
            with open(src, "w") as f:
                f.write(text)
            back = os.path.join(tmp, name + ".csr")
            run("read-mtx", src, back)
            brp, bci, bva, bcols = read_csr(back)
            store[name + "_read_rowptr"], store[name + "_read_col"], store[name + "_read_val"] = brp, bci, bva
            store[name + "_read_ncols"] = np.int64(bcols)
        # vectors
        rng = np.random.default_rng(5)
        for d, n in ((2, 25), (3, 125)):
            v = rng.standard_normal(n) * np.logspace(-8, 8, n)
            v[3] = 0.0
            v[4] = -1.0 / 3.0
            vb = os.path.join(tmp, "v%d.bin" % d)
            with open(vb, "wb") as f:
                f.write(struct.pack("<i", n))
                f.write(v.tobytes())
            vec = os.path.join(OUT, "vec%dd.vec" % d)
            run("write-vec", vb, os.path.join(tmp, "pos%d.bin" % d), vec)
            back = os.path.join(tmp, "v%d_back.bin" % d)
            run("read-vec", vec, str(n), back)
            store["vec%dd" % d] = v
            store["vec%dd_read" % d] = np.frombuffer(open(back, "rb").read()[4:], np.float64).copy()
            # WriteVector with a compare vector (SaveVectorDiffForConnectionViewer): v - w
            w = rng.standard_normal(n)
            wb = os.path.join(tmp, "w%d.bin" % d)
            with open(wb, "wb") as f:
                f.write(struct.pack("<i", n))
                f.write(w.tobytes())
            run("write-vec-diff", vb, wb, os.path.join(tmp, "pos%d.bin" % d), os.path.join(OUT, "vec%dd_diff.vec" % d))
            store["vec%dd_cmp" % d] = w
    np.savez(os.path.join(OUT, "cases.npz"), **store)
    print("wrote", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
