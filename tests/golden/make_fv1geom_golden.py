"""Generates tests/golden/fv1geom.npz from ugcore's own FV1 element geometry
and full-upwind convection shapes (oracle/_ref/ref_fv1geom, built by
oracle/build_ref.sh from the reference sources where they lie).

Contents, per element type t in quad, hex, tet, tri:
  e_<t>_*   seeded, distorted single elements: corners, K, and what ugcore's
            FV1Geometry computes for them (SCV volumes, SCVF from/to, area
            normals, integration points, shape gradients at the ips), the
            ConvectionShapesFullUpwind shapes for a velocity field evaluated
            at the ips, and the element matrix of -div(K grad u) + div(v u)
            assembled from them as the ConvectionDiffusion FV1 disc does;
  m_<t>_*   a small distorted mesh (structured cells with interior vertices
            moved, tets as 6 Kuhn tets per cell, triangles 2 per cell):
            coordinates, elements, log K per element, and the global
            operator before Dirichlet rows, with and without convection
            (dense; the mesh has at most a few hundred vertices).
The 3D velocity is v(x) = scale * sum_m -sin(k_m . x + phase_m) c_m (the
library's Fourier curl field); 2D cases have no convection.

Run here (where the reference tree is) with: python tests/golden/make_fv1geom_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_fv1geom")
TYPES = {"quad": (0, 2, 4), "hex": (1, 3, 8), "tet": (2, 3, 4), "tri": (3, 2, 3)}
NSCVF = {"quad": 4, "hex": 12, "tet": 6, "tri": 3}
REF = {
    "quad": [[0, 0], [1, 0], [1, 1], [0, 1]],
    "hex": [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
    "tet": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "tri": [[0, 0], [1, 0], [0, 1]],
}


def field(rng, dim):
    if dim == 2:
        return dict(k=np.zeros((0, 3)), c=np.zeros((0, 3)), phase=np.zeros(0), scale=0.0)
    nm = 4
    return dict(k=rng.uniform(-3, 3, (nm, 3)), c=rng.standard_normal((nm, 3)), phase=rng.uniform(0, 2 * np.pi, nm),
                scale=2.0)


def run(t, K, corners, F):
    code, dim, k = TYPES[t]
    lines = ["%d %d %d %.17g" % (code, len(K), len(F["phase"]), F["scale"])]
    for m in range(len(F["phase"])):
        lines.append(" ".join("%.17g" % v for v in list(F["k"][m]) + list(F["c"][m]) + [F["phase"][m]]))
    for e in range(len(K)):
        lines.append("%.17g " % K[e] + " ".join("%.17g" % v for v in corners[e].ravel()))
    r = subprocess.run([EXE], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    nf = NSCVF[t]
    out = dict(vol=[], frm=[], to=[], normal=[], ip=[], grad=[], up=[], A=[])
    cur = None
    for ln in r.stdout.splitlines():
        p = ln.split()
        if p[0] == "E":
            cur = dict(vol=None, frm=[], to=[], normal=[], ip=[], grad=[], up=[])
        elif p[0] == "S":
            cur["vol"] = [float(v) for v in p[1:]]
        elif p[0] == "F":
            v = [float(x) for x in p[3:]]
            cur["frm"].append(int(p[1]))
            cur["to"].append(int(p[2]))
            cur["normal"].append(v[:dim])
            cur["ip"].append(v[dim:2 * dim])
            cur["grad"].append(np.array(v[2 * dim:]).reshape(k, dim))
        elif p[0] == "U":
            cur["up"].append([float(x) for x in p[1:]])
        elif p[0] == "A":
            assert len(cur["frm"]) == nf
            for key in ("vol", "frm", "to", "normal", "ip", "grad", "up"):
                out[key].append(cur[key])
            out["A"].append(np.array([float(x) for x in p[1:]]).reshape(k, k))
    assert len(out["A"]) == len(K)
    return {key: np.array(v) for key, v in out.items()}


def orient(t, c):
    """positive orientation in ugcore's reference sense (swap two corners)"""
    if t == "tet":
        if np.linalg.det(np.array([c[1] - c[0], c[2] - c[0], c[3] - c[0]])) < 0:
            c[[1, 2]] = c[[2, 1]]
    elif t == "tri":
        d = c[1] - c[0], c[2] - c[0]
        if d[0][0] * d[1][1] - d[0][1] * d[1][0] < 0:
            c[[1, 2]] = c[[2, 1]]
    return c


def single_elements(rng, t, n=40):
    ref = np.array(REF[t], dtype=np.float64)
    dist = 0.18 if t in ("quad", "hex") else 0.25
    cs = []
    for _ in range(n):
        c = ref + rng.uniform(-dist, dist, ref.shape)
        c = c * rng.uniform(0.05, 2.0) + rng.uniform(-1, 1, ref.shape[1])
        cs.append(orient(t, c))
    return np.array(cs), np.exp(rng.standard_normal(n))


def mesh(rng, t):
    """structured cells with moved interior vertices; lexicographic vertices"""
    dim = TYPES[t][1]
    m = 5 if dim == 2 else 3
    n1 = m + 1
    if dim == 2:
        g = np.stack(np.meshgrid(np.arange(n1), np.arange(n1), indexing="xy"), -1).reshape(-1, 2).astype(float)
    else:
        z, y, x = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
        g = np.stack([x.ravel(), y.ravel(), z.ravel()], 1).astype(float)
    inner = np.all((g > 0) & (g < m), axis=1)
    coords = g / m
    coords[inner] += rng.uniform(-0.12, 0.12, (inner.sum(), dim)) / m

    def vid(*ix):
        return ix[0] + n1 * ix[1] + (n1 * n1 * ix[2] if dim == 3 else 0)
    elems = []
    if dim == 2:
        for j in range(m):
            for i in range(m):
                q = [vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)]
                if t == "quad":
                    elems.append(q)
                elif (i + j) % 2 == 0:
                    elems += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
                else:
                    elems += [[q[0], q[1], q[3]], [q[1], q[2], q[3]]]
    else:
        for kk in range(m):
            for j in range(m):
                for i in range(m):
                    h = [vid(i, j, kk), vid(i + 1, j, kk), vid(i + 1, j + 1, kk), vid(i, j + 1, kk),
                         vid(i, j, kk + 1), vid(i + 1, j, kk + 1), vid(i + 1, j + 1, kk + 1), vid(i, j + 1, kk + 1)]
                    if t == "hex":
                        elems.append(h)
                    else:
                        # 6 tets around the main diagonal 0-6 (corner bits x, y, z)
                        bits = {0: h[0], 1: h[1], 3: h[2], 2: h[3], 4: h[4], 5: h[5], 7: h[6], 6: h[7]}
                        for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
                            a = 0
                            path = [bits[0]]
                            for ax in perm:
                                a |= 1 << ax
                                path.append(bits[a])
                            elems.append(path)
    elems = np.array(elems, dtype=np.int32)
    for e in range(len(elems)):
        c = coords[elems[e]].copy()
        c2 = orient(t, c.copy())
        if not np.array_equal(c, c2):
            elems[e][[1, 2]] = elems[e][[2, 1]]
    return coords, elems


def assemble(t, coords, elems, res):
    n = len(coords)
    A = np.zeros((n, n))
    for e, el in enumerate(elems):
        A[np.ix_(el, el)] += res["A"][e]
    return A


def main():
    if not os.path.exists(EXE):
        sys.exit("build oracle/_ref/ref_fv1geom first (sh oracle/build_ref.sh)")
    rng = np.random.default_rng(2024)
    out = {}
    for t in TYPES:
        dim = TYPES[t][1]
        F = field(rng, dim)
        cs, K = single_elements(rng, t)
        r = run(t, K, cs, F)
        out["e_%s_corners" % t], out["e_%s_K" % t] = cs, K
        for key, v in r.items():
            out["e_%s_%s" % (t, key)] = v
        for key, v in F.items():
            out["e_%s_vel_%s" % (t, key)] = np.asarray(v)
        coords, elems = mesh(rng, t)
        mlog = rng.standard_normal(len(elems))
        Fm = field(rng, dim)
        rm = run(t, np.exp(mlog), coords[elems], Fm)
        F0 = dict(Fm, scale=0.0)
        r0 = run(t, np.exp(mlog), coords[elems], F0)
        out["m_%s_coords" % t], out["m_%s_elems" % t], out["m_%s_logK" % t] = coords, elems, mlog
        out["m_%s_A" % t] = assemble(t, coords, elems, rm)
        out["m_%s_A_diffusion" % t] = assemble(t, coords, elems, r0)
        for key, v in Fm.items():
            out["m_%s_vel_%s" % (t, key)] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "fv1geom.npz"), **out)
    print("wrote", os.path.join(HERE, "fv1geom.npz"))


if __name__ == "__main__":
    main()
