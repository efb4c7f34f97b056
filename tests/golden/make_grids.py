"""Writes the small unstructured coarse grids in golden/grids/ as UGX files
(the XML layout lib_grid/file_io/file_io_ugx.cpp reads: <vertices coords>,
<edges>, <triangles> / <quadrilaterals>, <tetrahedrons> / <hexahedrons>, and a
subset_handler whose subsets list vertex, edge, face and volume indices).

    square_tris.ugx   unit square, 8 triangles around an off-centre vertex;
                      subsets Inner, Dirichlet (the side x = 0), Neumann
    square_quads.ugx  unit square, 2 x 2 quadrilaterals, moved centre vertex;
                      subsets Inner, Boundary
    cube_tets.ugx     unit cube, 12 tetrahedra around an off-centre vertex;
                      subsets Inner, Bottom (z = 0), Other
    cube_hexes.ugx    unit cube, 2 x 2 x 2 hexahedra, moved centre vertex;
                      subsets Inner, Boundary

Usage: python tests/golden/make_grids.py
"""
import itertools
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "grids")


def fmt(a):
    return " ".join(repr(float(x)) if isinstance(x, (float, np.floating)) else str(int(x)) for x in np.ravel(a))


def write_ugx(path, coords, edges, faces, face_tag, vols, vol_tag, subsets):
    """subsets: [(name, vertex ids, edge ids, face ids, volume ids)]"""
    c3 = np.zeros((len(coords), 3))
    c3[:, :np.shape(coords)[1]] = coords
    lines = ['<?xml version="1.0" encoding="utf-8"?>', '<grid name="defGrid">',
             '\t<vertices coords="3">%s</vertices>' % fmt(c3),
             '\t<edges>%s</edges>' % fmt(edges)]
    if len(faces):
        lines.append('\t<%s>%s</%s>' % (face_tag, fmt(faces), face_tag))
    if len(vols):
        lines.append('\t<%s>%s</%s>' % (vol_tag, fmt(vols), vol_tag))
    lines.append('\t<subset_handler name="defSH">')
    for i, (name, sv, se, sf, svol) in enumerate(subsets):
        lines.append('\t\t<subset name="%s" color="%d 0 0 1" state="0">' % (name, i))
        for tag, ids in (("vertices", sv), ("edges", se), ("faces", sf), ("volumes", svol)):
            if len(ids):
                lines.append('\t\t\t<%s>%s</%s>' % (tag, fmt(sorted(ids)), tag))
        lines.append('\t\t</subset>')
    lines.append('\t</subset_handler>')
    lines.append('</grid>')
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def edge_list(cells, local_edges):
    es = []
    for c in cells:
        for a, b in local_edges:
            e = tuple(sorted((c[a], c[b])))
            if e not in es:
                es.append(e)
    return es


def square_tris():
    X = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [.5, 0], [1, .5], [.5, 1], [0, .5], [.4, .55]])
    ring = [0, 4, 1, 5, 2, 6, 3, 7]
    tris = [(ring[i], ring[(i + 1) % 8], 8) for i in range(8)]
    edges = edge_list(tris, [(0, 1), (1, 2), (2, 0)])
    left = [i for i, e in enumerate(edges) if X[e[0], 0] == 0 and X[e[1], 0] == 0]
    bnd = [i for i, e in enumerate(edges) if 8 not in e]
    inner = [i for i, e in enumerate(edges) if 8 in e]
    subsets = [("Inner", [8], inner, list(range(8)), []),
               ("Dirichlet", [0, 7, 3], left, [], []),
               ("Neumann", [4, 1, 5, 2, 6], [i for i in bnd if i not in left], [], [])]
    write_ugx(os.path.join(OUT, "square_tris.ugx"), X, edges, tris, "triangles", [], "", subsets)


def square_quads():
    X = np.array([[x, y] for y in (0, .5, 1) for x in (0, .5, 1)], dtype=float)
    X[4] = [.45, .55]
    quads = [(0, 1, 4, 3), (1, 2, 5, 4), (3, 4, 7, 6), (4, 5, 8, 7)]
    edges = edge_list(quads, [(0, 1), (1, 2), (2, 3), (3, 0)])
    bnd = [i for i, e in enumerate(edges) if 4 not in e]
    subsets = [("Inner", [4], [i for i in range(len(edges)) if i not in bnd], list(range(4)), []),
               ("Boundary", [v for v in range(9) if v != 4], bnd, [], [])]
    write_ugx(os.path.join(OUT, "square_quads.ugx"), X, edges, quads, "quadrilaterals", [], "", subsets)


CUBE = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
CUBE_FACES = [(0, 3, 2, 1), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]


def cube_tets():
    X = np.vstack([CUBE, [[.45, .5, .55]]])
    tris = []
    for q in CUBE_FACES:
        tris += [(q[0], q[1], q[2]), (q[0], q[2], q[3])]
    tets = [t + (8,) for t in tris]
    edges = edge_list(tets, [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)])
    bottom_f = [i for i, t in enumerate(tris) if all(X[v, 2] == 0 for v in t)]
    bottom_e = [i for i, e in enumerate(edges) if X[e[0], 2] == 0 and X[e[1], 2] == 0]
    bnd_e = [i for i, e in enumerate(edges) if 8 not in e]
    subsets = [("Inner", [8], [i for i, e in enumerate(edges) if 8 in e], [], list(range(len(tets)))),
               ("Bottom", [0, 1, 2, 3], bottom_e, bottom_f, []),
               ("Other", [4, 5, 6, 7], [i for i in bnd_e if i not in bottom_e],
                [i for i in range(len(tris)) if i not in bottom_f], [])]
    write_ugx(os.path.join(OUT, "cube_tets.ugx"), X, edges, tris, "triangles", tets, "tetrahedrons", subsets)


def cube_hexes():
    idx = {}
    X = []
    for z, y, x in itertools.product((0, .5, 1), repeat=3):
        idx[(x, y, z)] = len(X)
        X.append([x, y, z])
    X = np.array(X, float)
    centre = idx[(.5, .5, .5)]
    X[centre] = [.45, .55, .5]
    hexes = []
    for oz, oy, ox in itertools.product((0, .5), repeat=3):
        hexes.append(tuple(idx[(ox + .5 * c[0], oy + .5 * c[1], oz + .5 * c[2])] for c in CUBE))
    edges = edge_list(hexes, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (5, 6),
                              (6, 7), (7, 4)])
    on_bnd = [bool(np.any((X[v] == 0) | (X[v] == 1))) for v in range(len(X))]
    quads = []
    for h in hexes:
        for f in CUBE_FACES:
            q = tuple(h[j] for j in f)
            if all(on_bnd[v] for v in q) and any(np.all(X[list(q), d] == X[q[0], d]) and X[q[0], d] in (0, 1)
                                                for d in range(3)):
                quads.append(q)
    bnd_e = [i for i, e in enumerate(edges) if any(set(e) <= set(q) for q in quads)]
    subsets = [("Inner", [v for v in range(len(X)) if not on_bnd[v]],
                [i for i in range(len(edges)) if i not in bnd_e], [], list(range(len(hexes)))),
               ("Boundary", [v for v in range(len(X)) if on_bnd[v]], bnd_e, list(range(len(quads))), [])]
    write_ugx(os.path.join(OUT, "cube_hexes.ugx"), X, edges, quads, "quadrilaterals", hexes, "hexahedrons",
              subsets)


def main():
    os.makedirs(OUT, exist_ok=True)
    square_tris()
    square_quads()
    cube_tets()
    cube_hexes()
    print("wrote", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
