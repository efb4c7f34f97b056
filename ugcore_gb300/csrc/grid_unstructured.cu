// grid_unstructured.cu -- multigrid hierarchies of unstructured coarse grids.
//
// A coarse grid (from a UGX file or from arrays) is refined regularly, as
// GlobalMultiGridRefiner does (lib_grid/refinement/global_multi_grid_refiner.h,
// regular refinement rules of lib_grid/refinement/refinement_rules and
// tetrahedron_rules.cpp):
//   triangle      -> 4 (edge mid points),
//   quadrilateral -> 4 (edge mid points + centre),
//   tetrahedron   -> 8 (4 corner tets + the inner octahedron cut along its
//                   shortest diagonal; ties go to the first of (01,23),
//                   (12,03), (02,13)),
//   hexahedron    -> 8 (edge mid points, face centres, centre).
// New vertices sit at the averages of their parent object's corners (taken in
// increasing vertex index), and list those corners as their parents: the P1
// prolongation of StdTransfer (std_transfer_impl.h:47-168) then has the
// weights 1, 1/2, 1/4, 1/8 of the structured hierarchy.
//
// Vertex numbering of level l+1: the vertices of level l, then one per edge
// of level l (edges ordered by (smaller, larger) vertex index), then one per
// quadrilateral face (hexahedra: faces ordered by their sorted corners; 2D
// quadrilaterals: element order), then one per hexahedron.  Elements: the
// children of element 0, then of element 1, ...  Every element is stored with
// positive orientation (a negatively oriented coarse element has two corners
// swapped), which the FV1 geometry's area normals assume.
//
// Dirichlet vertices follow subset membership as in ugcore (a vertex
// created on an edge / face / element belongs to that object's subset; the
// children of an edge / face / element, and the edges and faces created
// inside it, inherit its subset): the grid keeps the edges, faces and
// elements of the Dirichlet subsets and refines those lists with the grid.
// Without subsets, the topological boundary (facets of one element) is the
// Dirichlet boundary.
//
// refine() below is the host statement of these rules (it also serves the
// host-only ug4gb_io_ugx_level); the hierarchies the solvers use are refined
// on the device by grid_refine_device.cu with the same numbering and the same
// (explicitly rounded) arithmetic.  A greedy element colouring (in index
// order) gives the assembly its race-free scatter order; the colour-ordered
// smoothers colour each level's operator graph themselves.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gmg.cuh"
#include "grid_refine.cuh"

namespace ug4gb {

namespace {

struct HostLevel {
    int elem_type = 0, dim = 2, k = 3, nv = 0, ne = 0;
    std::vector<double> coords;            // nv * dim
    std::vector<int> elems;                // ne * k
    std::vector<unsigned char> vdir;       // Dirichlet vertices
    std::vector<std::array<int, 2>> dir_edges;        // edges of Dirichlet subsets (a < b)
    std::vector<std::array<int, 4>> dir_faces;        // faces of Dirichlet subsets, cyclic order (-1: triangle)
    std::vector<unsigned char> edir;       // elements of Dirichlet subsets
    std::vector<int> npar, par;            // parents in the coarser level (par: nv * 8)
};

[[noreturn]] void fail(const std::string &m) { throw Error{UG4GB_ERR_INVALID, m}; }

int dim_of(int t) { return (t == UG4GB_QUAD || t == UG4GB_TRI) ? 2 : 3; }
int corners_of(int t) { return t == UG4GB_HEX ? 8 : (t == UG4GB_TRI ? 3 : 4); }

// reference-element edges (reference_element.cpp)
const int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kQuadEdges[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
const int kTetEdges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
const int kHexEdges[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5},
                              {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
const int kTetFaces[4][3] = {{0, 2, 1}, {1, 2, 3}, {0, 3, 2}, {0, 1, 3}};
const int kHexFaces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
// reference coordinates of the quadrilateral / hexahedron corners
const int kQuadRef[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
const int kHexRef[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

int num_edges(int t) { return t == UG4GB_TRI ? 3 : (t == UG4GB_QUAD ? 4 : (t == UG4GB_TET ? 6 : 12)); }
const int (*edges_of(int t))[2]
{
    return t == UG4GB_TRI ? kTriEdges : (t == UG4GB_QUAD ? kQuadEdges : (t == UG4GB_TET ? kTetEdges : kHexEdges));
}

// Unique keys grouped by their smallest vertex: ids in (first, rest) order.
// Used for edges (rest = 1 vertex) and quadrilateral faces (rest = 3).
template <int R>
struct KeyIndex {
    std::vector<int> off;                      // per first vertex
    std::vector<std::array<int, R>> rest;      // sorted within each first vertex
    void build(int nv, const std::vector<std::array<int, R + 1>> &keys)
    {
        off.assign((size_t)nv + 1, 0);
        for (const auto &k : keys) ++off[(size_t)k[0] + 1];
        for (int v = 0; v < nv; ++v) off[v + 1] += off[v];
        std::vector<int> cur(off.begin(), off.end() - 1);
        std::vector<std::array<int, R>> tmp(keys.size());
        for (const auto &k : keys) {
            std::array<int, R> r;
            for (int j = 0; j < R; ++j) r[j] = k[j + 1];
            tmp[cur[k[0]]++] = r;
        }
        rest.clear();
        std::vector<int> noff((size_t)nv + 1, 0);
        for (int v = 0; v < nv; ++v) {
            auto b = tmp.begin() + off[v], e = tmp.begin() + off[v + 1];
            std::sort(b, e);
            auto u = std::unique(b, e);
            rest.insert(rest.end(), b, u);
            noff[v + 1] = (int)rest.size();
        }
        off.swap(noff);
    }
    int size() const { return (int)rest.size(); }
    int find(const std::array<int, R + 1> &k) const
    {
        std::array<int, R> r;
        for (int j = 0; j < R; ++j) r[j] = k[j + 1];
        auto b = rest.begin() + off[k[0]], e = rest.begin() + off[k[0] + 1];
        auto it = std::lower_bound(b, e, r);
        return (it != e && *it == r) ? (int)(it - rest.begin()) : -1;
    }
};

std::array<int, 2> ekey(int a, int b) { return a < b ? std::array<int, 2>{a, b} : std::array<int, 2>{b, a}; }
std::array<int, 4> qkey(const int *q)
{
    std::array<int, 4> k{q[0], q[1], q[2], q[3]};
    std::sort(k.begin(), k.end());
    return k;
}
// 2D: twice the signed area of (ev[0], ev[1], ev[2]); 3D: six times the
// signed volume of (ev[0], ev[1], ev[2], ev[3])
double signed_measure(const HostLevel &L, const int *ev)
{
    const double *x0 = &L.coords[(size_t)ev[0] * L.dim], *x1 = &L.coords[(size_t)ev[1] * L.dim];
    const double *x2 = &L.coords[(size_t)ev[2] * L.dim];
    if (L.dim == 2) return (x1[0] - x0[0]) * (x2[1] - x0[1]) - (x1[1] - x0[1]) * (x2[0] - x0[0]);
    const double *x3 = &L.coords[(size_t)ev[3] * L.dim];
    const double a[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
    const double b[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
    const double c[3] = {x3[0] - x0[0], x3[1] - x0[1], x3[2] - x0[2]};
    return a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

// positive orientation: swap corners (simplices 1 <-> 2; quadrilateral 1 <-> 3;
// hexahedron bottom and top faces reversed alike)
void orient(HostLevel &L)
{
    for (int e = 0; e < L.ne; ++e) {
        int *ev = &L.elems[(size_t)e * L.k];
        if (L.elem_type == UG4GB_HEX) {
            // orientation of corner 0's frame (1 - 0, 3 - 0, 4 - 0)
            int f[4] = {ev[0], ev[1], ev[3], ev[4]};
            if (signed_measure(L, f) >= 0.0) continue;
            std::swap(ev[1], ev[3]);
            std::swap(ev[5], ev[7]);
        } else if (L.elem_type == UG4GB_QUAD) {
            if (signed_measure(L, ev) >= 0.0) continue;
            std::swap(ev[1], ev[3]);
        } else {
            if (signed_measure(L, ev) >= 0.0) continue;
            std::swap(ev[1], ev[2]);
        }
    }
}

// Dirichlet objects of the topological boundary (facets of one element)
void boundary_as_dirichlet(HostLevel &L)
{
    if (L.dim == 2) {
        std::vector<std::array<int, 3>> keys;
        const int ned = num_edges(L.elem_type);
        const int (*E)[2] = edges_of(L.elem_type);
        for (int e = 0; e < L.ne; ++e)
            for (int j = 0; j < ned; ++j) {
                auto k = ekey(L.elems[(size_t)e * L.k + E[j][0]], L.elems[(size_t)e * L.k + E[j][1]]);
                keys.push_back({k[0], k[1], 0});
            }
        std::sort(keys.begin(), keys.end());
        for (size_t i = 0; i < keys.size();) {
            size_t j = i;
            while (j < keys.size() && keys[j][0] == keys[i][0] && keys[j][1] == keys[i][1]) ++j;
            if (j - i == 1) L.dir_edges.push_back({keys[i][0], keys[i][1]});
            i = j;
        }
    } else {
        std::vector<std::array<int, 8>> keys;   // sorted corners (4, -1 padded) + cyclic corners
        const bool hex = L.elem_type == UG4GB_HEX;
        for (int e = 0; e < L.ne; ++e) {
            const int *ev = &L.elems[(size_t)e * L.k];
            for (int f = 0; f < (hex ? 6 : 4); ++f) {
                int q[4] = {-1, -1, -1, -1};
                for (int j = 0; j < (hex ? 4 : 3); ++j) q[j] = ev[hex ? kHexFaces[f][j] : kTetFaces[f][j]];
                std::array<int, 4> s{q[0], q[1], q[2], q[3]};
                std::sort(s.begin(), s.end());
                keys.push_back({s[0], s[1], s[2], s[3], q[0], q[1], q[2], q[3]});
            }
        }
        std::sort(keys.begin(), keys.end(), [](const std::array<int, 8> &a, const std::array<int, 8> &b) {
            return std::lexicographical_compare(a.begin(), a.begin() + 4, b.begin(), b.begin() + 4);
        });
        for (size_t i = 0; i < keys.size();) {
            size_t j = i;
            while (j < keys.size() && std::equal(keys[j].begin(), keys[j].begin() + 4, keys[i].begin())) ++j;
            if (j - i == 1) L.dir_faces.push_back({keys[i][4], keys[i][5], keys[i][6], keys[i][7]});
            i = j;
        }
        for (const auto &f : L.dir_faces) {
            const int n = f[3] < 0 ? 3 : 4;
            for (int j = 0; j < n; ++j) L.dir_edges.push_back(ekey(f[j], f[(j + 1) % n]));
        }
    }
    for (const auto &e : L.dir_edges) L.vdir[e[0]] = L.vdir[e[1]] = 1;
    for (const auto &f : L.dir_faces)
        for (int j = 0; j < 4; ++j)
            if (f[j] >= 0) L.vdir[f[j]] = 1;
}

void dedupe(HostLevel &L)
{
    std::sort(L.dir_edges.begin(), L.dir_edges.end());
    L.dir_edges.erase(std::unique(L.dir_edges.begin(), L.dir_edges.end()), L.dir_edges.end());
    // faces: unique by their sorted corners (first cyclic order kept)
    std::vector<std::pair<std::array<int, 4>, std::array<int, 4>>> fs;
    for (const auto &f : L.dir_faces) {
        std::array<int, 4> s = f;
        std::sort(s.begin(), s.end());
        fs.push_back({s, f});
    }
    std::stable_sort(fs.begin(), fs.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    L.dir_faces.clear();
    for (size_t i = 0; i < fs.size(); ++i)
        if (i == 0 || fs[i].first != fs[i - 1].first) L.dir_faces.push_back(fs[i].second);
}

// one regular refinement step
void refine(const HostLevel &C, HostLevel &F)
{
    const int t = C.elem_type, k = C.k, dim = C.dim, ned = num_edges(t);
    const int (*E)[2] = edges_of(t);
    // edges
    KeyIndex<1> edges;
    {
        std::vector<std::array<int, 2>> keys;
        keys.reserve((size_t)C.ne * ned);
        for (int e = 0; e < C.ne; ++e)
            for (int j = 0; j < ned; ++j)
                keys.push_back(ekey(C.elems[(size_t)e * k + E[j][0]], C.elems[(size_t)e * k + E[j][1]]));
        edges.build(C.nv, keys);
    }
    const int nedge = edges.size();
    // quadrilateral faces of hexahedra
    KeyIndex<3> qfaces;
    if (t == UG4GB_HEX) {
        std::vector<std::array<int, 4>> keys;
        keys.reserve((size_t)C.ne * 6);
        for (int e = 0; e < C.ne; ++e)
            for (int f = 0; f < 6; ++f) {
                int q[4];
                for (int j = 0; j < 4; ++j) q[j] = C.elems[(size_t)e * k + kHexFaces[f][j]];
                keys.push_back(qkey(q));
            }
        qfaces.build(C.nv, keys);
    }
    const int nqf = (t == UG4GB_HEX) ? qfaces.size() : (t == UG4GB_QUAD ? C.ne : 0);
    const int ncen = (t == UG4GB_HEX) ? C.ne : 0;
    const int64_t nv64 = (int64_t)C.nv + nedge + nqf + ncen;
    if (nv64 >= ((int64_t)1 << 31)) fail("refinement: too many vertices for 32-bit indices");
    const int64_t ne64 = (int64_t)C.ne * (dim == 2 ? 4 : 8);
    if (ne64 * k >= ((int64_t)1 << 31)) fail("refinement: too many elements for 32-bit indices");
    F.elem_type = t;
    F.dim = dim;
    F.k = k;
    F.nv = (int)nv64;
    F.ne = (int)ne64;
    F.coords.assign((size_t)F.nv * dim, 0.0);
    F.vdir.assign(F.nv, 0);
    F.npar.assign(F.nv, 0);
    F.par.assign((size_t)F.nv * 8, -1);
    auto set_vertex = [&](int v, const int *corners, int n) {
        int s[8];
        std::copy(corners, corners + n, s);
        std::sort(s, s + n);
        for (int d = 0; d < dim; ++d) {
            double acc = 0.0;
            for (int j = 0; j < n; ++j) acc += C.coords[(size_t)s[j] * dim + d];
            F.coords[(size_t)v * dim + d] = acc * (1.0 / n);
        }
        F.npar[v] = n;
        for (int j = 0; j < n; ++j) F.par[(size_t)v * 8 + j] = s[j];
    };
    for (int v = 0; v < C.nv; ++v) {
        set_vertex(v, &v, 1);
        F.vdir[v] = C.vdir[v];
    }
    for (int a = 0; a < C.nv; ++a)
        for (int i = edges.off[a]; i < edges.off[a + 1]; ++i) {
            int c2[2] = {a, edges.rest[i][0]};
            set_vertex(C.nv + i, c2, 2);
        }
    if (t == UG4GB_HEX) {
        for (int a = 0; a < C.nv; ++a)
            for (int i = qfaces.off[a]; i < qfaces.off[a + 1]; ++i) {
                int c4[4] = {a, qfaces.rest[i][0], qfaces.rest[i][1], qfaces.rest[i][2]};
                set_vertex(C.nv + nedge + i, c4, 4);
            }
        for (int e = 0; e < C.ne; ++e) set_vertex(C.nv + nedge + nqf + e, &C.elems[(size_t)e * k], 8);
    } else if (t == UG4GB_QUAD) {
        for (int e = 0; e < C.ne; ++e) set_vertex(C.nv + nedge + e, &C.elems[(size_t)e * k], 4);
    }
    auto mid = [&](int a, int b) {
        const int i = edges.find(ekey(a, b));
        if (i < 0) fail("refinement: edge not found");
        return C.nv + i;
    };
    auto qcentre = [&](const int *q) {
        const int i = qfaces.find(qkey(q));
        if (i < 0) fail("refinement: face not found");
        return C.nv + nedge + i;
    };
    // Dirichlet vertices from the objects of the Dirichlet subsets
    for (const auto &de : C.dir_edges) F.vdir[mid(de[0], de[1])] = 1;
    // children
    F.elems.assign((size_t)F.ne * k, -1);
    F.edir.assign(F.ne, 0);
    std::vector<std::array<int, 2>> inner_edges;   // created inside Dirichlet elements
    std::vector<std::array<int, 4>> inner_faces;
    for (int e = 0; e < C.ne; ++e) {
        const int *ev = &C.elems[(size_t)e * k];
        int *out = &F.elems[(size_t)e * (dim == 2 ? 4 : 8) * k];
        const bool ed = C.edir[e] != 0;
        for (int q = 0; q < (dim == 2 ? 4 : 8); ++q) F.edir[(size_t)e * (dim == 2 ? 4 : 8) + q] = C.edir[e];
        if (t == UG4GB_TRI) {
            const int m0 = mid(ev[0], ev[1]), m1 = mid(ev[1], ev[2]), m2 = mid(ev[2], ev[0]);
            const int ch[4][3] = {{ev[0], m0, m2}, {m0, ev[1], m1}, {m2, m1, ev[2]}, {m0, m1, m2}};
            for (int q = 0; q < 4; ++q)
                for (int j = 0; j < 3; ++j) out[q * 3 + j] = ch[q][j];
            if (ed) {
                inner_edges.push_back(ekey(m0, m1));
                inner_edges.push_back(ekey(m1, m2));
                inner_edges.push_back(ekey(m2, m0));
                F.vdir[m0] = F.vdir[m1] = F.vdir[m2] = 1;
            }
        } else if (t == UG4GB_TET) {
            const int m01 = mid(ev[0], ev[1]), m12 = mid(ev[1], ev[2]), m02 = mid(ev[0], ev[2]);
            const int m03 = mid(ev[0], ev[3]), m13 = mid(ev[1], ev[3]), m23 = mid(ev[2], ev[3]);
            const int corner[4][4] = {{ev[0], m01, m02, m03}, {m01, ev[1], m12, m13}, {m02, m12, ev[2], m23},
                                      {m03, m13, m23, ev[3]}};
            for (int q = 0; q < 4; ++q)
                for (int j = 0; j < 4; ++j) out[q * 4 + j] = corner[q][j];
            // octahedron: diagonals and the cycles of the other four around them
            const int diag[3][2] = {{m01, m23}, {m12, m03}, {m02, m13}};
            const int ring[3][4] = {{m12, m13, m03, m02}, {m01, m13, m23, m02}, {m01, m12, m23, m03}};
            int best = 0;
            double bl = 0.0;
            for (int d = 0; d < 3; ++d) {
                double l2 = 0.0;
                for (int x = 0; x < 3; ++x) {
                    const double dd = F.coords[(size_t)diag[d][0] * 3 + x] - F.coords[(size_t)diag[d][1] * 3 + x];
                    l2 += dd * dd;
                }
                if (d == 0 || l2 < bl) {
                    bl = l2;
                    best = d;
                }
            }
            for (int q = 0; q < 4; ++q) {
                int *o = out + (4 + q) * 4;
                o[0] = diag[best][0];
                o[1] = diag[best][1];
                o[2] = ring[best][q];
                o[3] = ring[best][(q + 1) % 4];
            }
            if (ed) {
                inner_edges.push_back(ekey(diag[best][0], diag[best][1]));
                for (int q = 0; q < 4; ++q) {
                    inner_faces.push_back({diag[best][0], diag[best][1], ring[best][q], -1});
                    const int *c = corner[q];
                    // the inner face of corner tet q: its three edge mid points
                    int fm[3], n = 0;
                    for (int j = 0; j < 4; ++j)
                        if (c[j] != ev[q]) fm[n++] = c[j];
                    inner_faces.push_back({fm[0], fm[1], fm[2], -1});
                }
                const int ms[6] = {m01, m12, m02, m03, m13, m23};
                for (int j = 0; j < 6; ++j) F.vdir[ms[j]] = 1;
            }
        } else {
            // quadrilateral / hexahedron: tensor sub-boxes; the point of child
            // corner j is the parent object spanned by the coordinates that
            // are 1/2 (corner, edge mid point, face centre or centre)
            const int nd = dim, nch = 1 << nd;
            for (int q = 0; q < nch; ++q)
                for (int j = 0; j < k; ++j) {
                    int h[3];
                    for (int d = 0; d < nd; ++d) {
                        const int o = (q >> d) & 1;
                        const int r = (nd == 2) ? kQuadRef[j][d] : kHexRef[j][d];
                        h[d] = o + r;   // 0, 1, 2 in half units
                    }
                    int cs[8], n = 0;
                    for (int i = 0; i < k; ++i) {
                        bool in = true;
                        for (int d = 0; d < nd; ++d) {
                            const int r = 2 * ((nd == 2) ? kQuadRef[i][d] : kHexRef[i][d]);
                            if (h[d] != 1 && h[d] != r) in = false;
                        }
                        if (in) cs[n++] = ev[i];
                    }
                    int v;
                    if (n == 1) v = cs[0];
                    else if (n == 2) v = mid(cs[0], cs[1]);
                    else if (n == 4) v = (t == UG4GB_QUAD) ? C.nv + nedge + e : qcentre(cs);
                    else v = C.nv + nedge + nqf + e;
                    out[q * k + j] = v;
                }
            if (ed) {
                for (int j = 0; j < ned; ++j) F.vdir[mid(ev[E[j][0]], ev[E[j][1]])] = 1;
                if (t == UG4GB_QUAD) {
                    const int z = C.nv + nedge + e;
                    F.vdir[z] = 1;
                    for (int j = 0; j < 4; ++j) inner_edges.push_back(ekey(z, mid(ev[E[j][0]], ev[E[j][1]])));
                } else {
                    const int z = C.nv + nedge + nqf + e;
                    F.vdir[z] = 1;
                    for (int f = 0; f < 6; ++f) {
                        int qf[4];
                        for (int j = 0; j < 4; ++j) qf[j] = ev[kHexFaces[f][j]];
                        const int fc = qcentre(qf);
                        F.vdir[fc] = 1;
                        inner_edges.push_back(ekey(z, fc));
                    }
                    // the 12 inner faces: centre, face centres and edge mid points
                    for (int j = 0; j < 12; ++j) {
                        int a = ev[E[j][0]], b = ev[E[j][1]];
                        const int m = mid(a, b);
                        int fcs[2], n = 0;
                        for (int f = 0; f < 6 && n < 2; ++f) {
                            int has = 0;
                            for (int x = 0; x < 4; ++x) has += (kHexFaces[f][x] == E[j][0] || kHexFaces[f][x] == E[j][1]);
                            if (has == 2) {
                                int qf[4];
                                for (int x = 0; x < 4; ++x) qf[x] = ev[kHexFaces[f][x]];
                                fcs[n++] = qcentre(qf);
                            }
                        }
                        inner_faces.push_back({m, fcs[0], z, fcs[1]});
                    }
                }
            }
        }
    }
    // Dirichlet objects of the fine level
    for (const auto &de : C.dir_edges) {
        const int m = mid(de[0], de[1]);
        F.dir_edges.push_back(ekey(de[0], m));
        F.dir_edges.push_back(ekey(m, de[1]));
    }
    for (const auto &df : C.dir_faces) {
        if (df[3] < 0) {
            const int a = df[0], b = df[1], c = df[2];
            const int mab = mid(a, b), mbc = mid(b, c), mca = mid(c, a);
            F.vdir[mab] = F.vdir[mbc] = F.vdir[mca] = 1;
            F.dir_edges.push_back(ekey(mab, mbc));
            F.dir_edges.push_back(ekey(mbc, mca));
            F.dir_edges.push_back(ekey(mca, mab));
            F.dir_faces.push_back({a, mab, mca, -1});
            F.dir_faces.push_back({mab, b, mbc, -1});
            F.dir_faces.push_back({mca, mbc, c, -1});
            F.dir_faces.push_back({mab, mbc, mca, -1});
        } else {
            const int *q = df.data();
            const int z = (t == UG4GB_HEX) ? qcentre(q) : -1;
            if (z < 0) fail("refinement: quadrilateral Dirichlet face in a grid without hexahedra");
            int m[4];
            for (int j = 0; j < 4; ++j) m[j] = mid(q[j], q[(j + 1) % 4]);
            F.vdir[z] = 1;
            for (int j = 0; j < 4; ++j) {
                F.vdir[m[j]] = 1;
                F.dir_edges.push_back(ekey(z, m[j]));
            }
            F.dir_faces.push_back({q[0], m[0], z, m[3]});
            F.dir_faces.push_back({m[0], q[1], m[1], z});
            F.dir_faces.push_back({z, m[1], q[2], m[2]});
            F.dir_faces.push_back({m[3], z, m[2], q[3]});
        }
    }
    F.dir_edges.insert(F.dir_edges.end(), inner_edges.begin(), inner_edges.end());
    F.dir_faces.insert(F.dir_faces.end(), inner_faces.begin(), inner_faces.end());
    orient(F);
    dedupe(F);
}

// greedy colouring in index order: elements, no shared vertex within a colour
void colour_elements(const HostLevel &L, std::vector<int> &off, std::vector<int> &list)
{
    const int W = 8;   // 512 colours at most
    std::vector<uint64_t> used((size_t)L.nv * W, 0);
    std::vector<int> col(L.ne);
    int ncol = 0;
    for (int e = 0; e < L.ne; ++e) {
        uint64_t m[W] = {0};
        const int *ev = &L.elems[(size_t)e * L.k];
        for (int i = 0; i < L.k; ++i)
            for (int w = 0; w < W; ++w) m[w] |= used[(size_t)ev[i] * W + w];
        int c = -1;
        for (int w = 0; w < W && c < 0; ++w)
            if (~m[w]) c = 64 * w + __builtin_ctzll(~m[w]);
        if (c < 0) fail("element colouring: more than 512 colours");
        col[e] = c;
        ncol = std::max(ncol, c + 1);
        for (int i = 0; i < L.k; ++i) used[(size_t)ev[i] * W + c / 64] |= 1ULL << (c % 64);
    }
    off.assign(ncol + 1, 0);
    for (int e = 0; e < L.ne; ++e) ++off[col[e] + 1];
    for (int c = 0; c < ncol; ++c) off[c + 1] += off[c];
    list.resize(L.ne);
    std::vector<int> cur(off.begin(), off.end() - 1);
    for (int e = 0; e < L.ne; ++e) list[cur[col[e]]++] = e;
}

void upload(Ctx &c, const HostLevel &H, Level &L)
{
    L.elem_type = H.elem_type;
    L.dim = H.dim;
    L.k = H.k;
    L.nv = H.nv;
    L.ne = H.ne;
    L.nx = L.ny = L.nz = 0;
    L.structured = false;
    L.coords.alloc(H.coords.size());
    L.elems.alloc(H.elems.size());
    L.bnd.alloc(H.nv);
    copy_in(c, L.coords.p, H.coords.data(), sizeof(double) * H.coords.size());
    copy_in(c, L.elems.p, H.elems.data(), sizeof(int) * H.elems.size());
    copy_in(c, L.bnd.p, H.vdir.data(), H.nv);
    if (!H.npar.empty()) {
        L.npar.alloc(H.nv);
        L.par.alloc((size_t)H.nv * 8);
        copy_in(c, L.npar.p, H.npar.data(), sizeof(int) * H.nv);
        copy_in(c, L.par.p, H.par.data(), sizeof(int) * H.par.size());
    }
    std::vector<int> list;
    colour_elements(H, L.ecol_off, list);
    L.ecol.alloc(std::max<size_t>(list.size(), 1));
    copy_in(c, L.ecol.p, list.data(), sizeof(int) * list.size());
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

void check_level0(HostLevel &L)
{
    if (L.elem_type < UG4GB_QUAD || L.elem_type > UG4GB_TRI) fail("grid: bad element type");
    L.dim = dim_of(L.elem_type);
    L.k = corners_of(L.elem_type);
    if (L.nv <= 0 || L.ne <= 0) fail("grid: no vertices or elements");
    if ((int64_t)L.elems.size() != (int64_t)L.ne * L.k || (int64_t)L.coords.size() != (int64_t)L.nv * L.dim)
        fail("grid: array sizes do not match");
    for (int v : L.elems)
        if (v < 0 || v >= L.nv) fail("grid: element corner out of range");
    if ((int)L.vdir.size() != L.nv) L.vdir.assign(L.nv, 0);
    if ((int)L.edir.size() != L.ne) L.edir.assign(L.ne, 0);
    orient(L);
    dedupe(L);
}

// ------------------------------------------------------------------- UGX --
// The parts of a UGX file (lib_grid/file_io/file_io_ugx.cpp, reader
// file_io_ugx_impl.hpp:440-520) the hierarchy needs: <vertices coords="d">,
// <edges>, <triangles>, <quadrilaterals>, <tetrahedrons>, <hexahedrons> (faces
// and volumes indexed in file order, as the reader appends them), and the
// subsets of the first <subset_handler> with their <vertices>, <edges>,
// <faces>, <volumes> index lists.
struct Ugx {
    int cdim = 0;
    std::vector<double> coords;
    std::vector<int> edges;
    std::vector<int> faces, face_n;      // corners (padded to 4), corner count
    std::vector<int> vols, vol_type;     // corners (padded to 8), UG4GB_TET / UG4GB_HEX
    struct Subset {
        std::string name;
        std::vector<int> v, e, f, vol;
    };
    std::vector<Subset> subsets;
};

std::string read_text(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) fail(std::string("UGX: cannot open ") + path);
    std::string s;
    char buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
    fclose(f);
    return s;
}

// content of the next element <name ...>...</name> at or after pos (empty
// element "<name .../>" gives an empty body); returns false if none
bool xml_element(const std::string &s, const std::string &name, size_t from, size_t to, size_t &body_b, size_t &body_e,
                 size_t &end, std::string *attrs = nullptr)
{
    size_t p = from;
    while (true) {
        p = s.find("<" + name, p);
        if (p == std::string::npos || p >= to) return false;
        const char nc = s[p + 1 + name.size()];
        if (nc == ' ' || nc == '>' || nc == '/' || nc == '\t' || nc == '\n' || nc == '\r') break;
        p += 1;
    }
    const size_t gt = s.find('>', p);
    if (gt == std::string::npos) fail("UGX: unterminated tag <" + name);
    if (attrs) *attrs = s.substr(p + 1 + name.size(), gt - p - 1 - name.size());
    if (s[gt - 1] == '/') {
        body_b = body_e = gt + 1;
        end = gt + 1;
        return true;
    }
    const size_t close = s.find("</" + name + ">", gt);
    if (close == std::string::npos) fail("UGX: missing </" + name + ">");
    body_b = gt + 1;
    body_e = close;
    end = close + name.size() + 3;
    return true;
}

std::string attr(const std::string &attrs, const std::string &key)
{
    const size_t p = attrs.find(key + "=\"");
    if (p == std::string::npos) return "";
    const size_t b = p + key.size() + 2, e = attrs.find('"', b);
    return attrs.substr(b, e - b);
}

template <class T>
void numbers(const std::string &s, size_t b, size_t e, std::vector<T> &out)
{
    const std::string t = s.substr(b, e - b);
    const char *c = t.c_str();
    char *end;
    while (true) {
        while (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r') ++c;
        if (!*c) break;
        const double v = strtod(c, &end);
        if (end == c) fail("UGX: bad number in list");
        out.push_back((T)v);
        c = end;
    }
}

Ugx parse_ugx(const char *path)
{
    const std::string s = read_text(path);
    Ugx U;
    size_t gb, ge, gend;
    if (!xml_element(s, "grid", 0, s.size(), gb, ge, gend)) fail("UGX: no <grid>");
    size_t b, e, end;
    std::string at;
    if (!xml_element(s, "vertices", gb, ge, b, e, end, &at)) fail("UGX: no <vertices>");
    U.cdim = atoi(attr(at, "coords").c_str());
    if (U.cdim < 1 || U.cdim > 3) fail("UGX: vertices coords attribute must be 1..3");
    numbers(s, b, e, U.coords);
    if (U.coords.size() % U.cdim) fail("UGX: vertex coordinate count");
    // grid element nodes in file order (faces / volumes are indexed that way)
    size_t p = gb;
    while (p < ge) {
        const size_t lt = s.find('<', p);
        if (lt == std::string::npos || lt >= ge) break;
        size_t nb = lt + 1, ne_ = nb;
        while (ne_ < s.size() && (isalnum((unsigned char)s[ne_]) || s[ne_] == '_')) ++ne_;
        const std::string name = s.substr(nb, ne_ - nb);
        if (name.empty()) {
            p = lt + 1;
            continue;
        }
        if (!xml_element(s, name, lt, ge, b, e, end)) break;
        std::vector<int> ids;
        if (name == "edges") {
            numbers(s, b, e, U.edges);
        } else if (name == "triangles" || name == "quadrilaterals") {
            const int n = name == "triangles" ? 3 : 4;
            numbers(s, b, e, ids);
            if (ids.size() % n) fail("UGX: " + name + " index count");
            for (size_t i = 0; i < ids.size(); i += n) {
                for (int j = 0; j < 4; ++j) U.faces.push_back(j < n ? ids[i + j] : -1);
                U.face_n.push_back(n);
            }
        } else if (name == "tetrahedrons" || name == "hexahedrons") {
            const int n = name == "tetrahedrons" ? 4 : 8;
            numbers(s, b, e, ids);
            if (ids.size() % n) fail("UGX: " + name + " index count");
            for (size_t i = 0; i < ids.size(); i += n) {
                for (int j = 0; j < 8; ++j) U.vols.push_back(j < n ? ids[i + j] : -1);
                U.vol_type.push_back(n == 4 ? UG4GB_TET : UG4GB_HEX);
            }
        } else if (name == "prisms" || name == "pyramids" || name == "octahedrons" ||
                   name.rfind("constrained", 0) == 0 || name.rfind("constraining", 0) == 0) {
            fail("UGX: " + name + " are not supported (triangles, quadrilaterals, tetrahedra, hexahedra are)");
        }
        p = end;
    }
    // first subset handler
    size_t sb, se, send;
    if (xml_element(s, "subset_handler", gb, ge, sb, se, send)) {
        size_t q = sb;
        while (xml_element(s, "subset", q, se, b, e, end, &at)) {
            Ugx::Subset S;
            S.name = attr(at, "name");
            size_t b2, e2, end2;
            if (xml_element(s, "vertices", b, e, b2, e2, end2)) numbers(s, b2, e2, S.v);
            if (xml_element(s, "edges", b, e, b2, e2, end2)) numbers(s, b2, e2, S.e);
            if (xml_element(s, "faces", b, e, b2, e2, end2)) numbers(s, b2, e2, S.f);
            if (xml_element(s, "volumes", b, e, b2, e2, end2)) numbers(s, b2, e2, S.vol);
            U.subsets.push_back(S);
            q = end;
        }
    }
    return U;
}

std::vector<std::string> split_names(const char *names)
{
    std::vector<std::string> out;
    if (!names) return out;
    std::string cur;
    for (const char *c = names;; ++c) {
        if (!*c || *c == ',') {
            size_t b = cur.find_first_not_of(' '), e = cur.find_last_not_of(' ');
            if (b != std::string::npos) out.push_back(cur.substr(b, e - b + 1));
            cur.clear();
            if (!*c) break;
        } else {
            cur += *c;
        }
    }
    return out;
}

// level 0 of a UGX grid; dirichlet: comma-separated subset names, NULL or
// "" = the topological boundary
HostLevel ugx_level0(const char *path, const char *dirichlet)
{
    const Ugx U = parse_ugx(path);
    HostLevel L;
    const int nv = (int)(U.coords.size() / U.cdim);
    const bool vol = !U.vol_type.empty();
    int type = -1;
    if (vol) {
        type = U.vol_type[0];
        for (int t : U.vol_type)
            if (t != type) fail("UGX: grids with more than one volume element type are not supported");
    } else {
        if (U.face_n.empty()) fail("UGX: no faces or volumes");
        for (int n : U.face_n)
            if (n != U.face_n[0]) fail("UGX: grids with both triangles and quadrilaterals are not supported");
        type = U.face_n[0] == 3 ? UG4GB_TRI : UG4GB_QUAD;
    }
    L.elem_type = type;
    L.dim = dim_of(type);
    L.k = corners_of(type);
    if (U.cdim < L.dim) fail("UGX: fewer coordinates than the element dimension");
    L.nv = nv;
    L.coords.resize((size_t)nv * L.dim);
    for (int v = 0; v < nv; ++v)
        for (int d = 0; d < L.dim; ++d) L.coords[(size_t)v * L.dim + d] = U.coords[(size_t)v * U.cdim + d];
    if (vol) {
        L.ne = (int)U.vol_type.size();
        for (int e = 0; e < L.ne; ++e)
            for (int j = 0; j < L.k; ++j) L.elems.push_back(U.vols[(size_t)e * 8 + j]);
    } else {
        L.ne = (int)U.face_n.size();
        for (int e = 0; e < L.ne; ++e)
            for (int j = 0; j < L.k; ++j) L.elems.push_back(U.faces[(size_t)e * 4 + j]);
    }
    L.vdir.assign(nv, 0);
    L.edir.assign(L.ne, 0);
    const std::vector<std::string> names = split_names(dirichlet);
    if (names.empty()) {
        check_level0(L);
        boundary_as_dirichlet(L);
        dedupe(L);
        return L;
    }
    for (const auto &nm : names) {
        const Ugx::Subset *S = nullptr;
        for (const auto &x : U.subsets)
            if (x.name == nm) S = &x;
        if (!S) fail("UGX: no subset named '" + nm + "'");
        for (int v : S->v) {
            if (v < 0 || v >= nv) fail("UGX: subset vertex out of range");
            L.vdir[v] = 1;
        }
        for (int i : S->e) {
            if (i < 0 || 2 * (size_t)i + 1 >= U.edges.size()) fail("UGX: subset edge out of range");
            L.dir_edges.push_back(ekey(U.edges[2 * i], U.edges[2 * i + 1]));
        }
        for (int i : S->f) {
            if (i < 0 || (size_t)i >= U.face_n.size()) fail("UGX: subset face out of range");
            if (vol) {
                std::array<int, 4> f{U.faces[(size_t)i * 4], U.faces[(size_t)i * 4 + 1], U.faces[(size_t)i * 4 + 2],
                                     U.face_n[i] == 4 ? U.faces[(size_t)i * 4 + 3] : -1};
                L.dir_faces.push_back(f);
            } else {
                L.edir[i] = 1;   // 2D: the face is an element
            }
        }
        for (int i : S->vol) {
            if (i < 0 || i >= L.ne || !vol) fail("UGX: subset volume out of range");
            L.edir[i] = 1;
        }
    }
    check_level0(L);
    return L;
}

}  // namespace

namespace {

// the Dirichlet objects of a host level, for the device refinement
void upload_dirichlet(Ctx &c, const HostLevel &H, DevDir &D)
{
    std::vector<u64> e(H.dir_edges.size());
    for (size_t i = 0; i < e.size(); ++i)
        e[i] = ((u64)(unsigned)H.dir_edges[i][0] << 32) | (u64)(unsigned)H.dir_edges[i][1];
    std::vector<int4> f(H.dir_faces.size());
    for (size_t i = 0; i < f.size(); ++i)
        f[i] = make_int4(H.dir_faces[i][0], H.dir_faces[i][1], H.dir_faces[i][2], H.dir_faces[i][3]);
    D.n_edges = (int)e.size();
    D.n_faces = (int)f.size();
    D.edges.alloc(std::max<size_t>(e.size(), 1));
    D.faces.alloc(std::max<size_t>(f.size(), 1));
    D.edir.alloc(std::max<size_t>(H.edir.size(), 1));
    copy_in(c, D.edges.p, e.data(), sizeof(u64) * e.size());
    copy_in(c, D.faces.p, f.data(), sizeof(int4) * f.size());
    copy_in(c, D.edir.p, H.edir.data(), H.edir.size());
}

// element colouring of a level refined on the device
void colour_level(Ctx &c, Level &L)
{
    HostLevel H;
    H.elem_type = L.elem_type;
    H.dim = L.dim;
    H.k = L.k;
    H.nv = L.nv;
    H.ne = L.ne;
    H.elems.resize((size_t)L.ne * L.k);
    copy_out(c, H.elems.data(), L.elems.p, sizeof(int) * H.elems.size());
    std::vector<int> list;
    colour_elements(H, L.ecol_off, list);
    L.ecol.alloc(std::max<size_t>(list.size(), 1));
    copy_in(c, L.ecol.p, list.data(), sizeof(int) * list.size());
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace

// Hierarchy of `nref` refinements of level 0: level 0 is uploaded, every
// finer level is refined on the device from the one below it (the same
// numbering and arithmetic as refine() above); only the greedy element colouring,
// sequential in index order, runs on the host.
void build_unstructured(Ctx &c, HostLevel L0, int nref, std::vector<Level> &lev)
{
    lev.clear();
    lev.resize(nref + 1);
    upload(c, L0, lev[0]);
    std::vector<DevDir> dir(nref + 1);
    upload_dirichlet(c, L0, dir[0]);
    for (int l = 1; l <= nref; ++l) {
        refine_device(c, lev[l - 1], dir[l - 1], lev[l], dir[l]);
        colour_level(c, lev[l]);
        dir[l - 1] = DevDir();
    }
}

}  // namespace ug4gb

using namespace ug4gb;

namespace {

template <class F>
int guarded(ug4gb_ctx *ctx, F &&f)
{
    try {
        f();
        return UG4GB_OK;
    } catch (const Error &e) {
        if (ctx) ctx->c.err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        if (ctx) ctx->c.err = "out of host memory";
        return UG4GB_ERR_NOMEM;
    }
}

int make_grid(ug4gb_ctx *ctx, HostLevel L0, int nref, ug4gb_grid **out)
{
    ug4gb_grid *g = new ug4gb_grid;
    const int rc = guarded(ctx, [&] {
        UG_REQUIRE(nref >= 0 && nref <= 10, UG4GB_ERR_INVALID, "grid: refinement count out of range");
        g->ctx = ctx;
        g->elem_type = L0.elem_type;
        build_unstructured(ctx->c, std::move(L0), nref, g->lev);
    });
    if (rc != UG4GB_OK) {
        delete g;
        return rc;
    }
    ug4gb_ctx_retain(ctx);
    *out = g;
    return UG4GB_OK;
}

}  // namespace

extern "C" {

int ug4gb_grid_create_ugx(ug4gb_ctx *ctx, const char *filename, int nref, const char *dirichlet_subsets,
                          ug4gb_grid **out)
{
    if (!ctx || !filename || !out) return UG4GB_ERR_INVALID;
    *out = nullptr;
    HostLevel L0;
    const int rc = guarded(ctx, [&] { L0 = ugx_level0(filename, dirichlet_subsets); });
    if (rc != UG4GB_OK) return rc;
    return make_grid(ctx, std::move(L0), nref, out);
}

int ug4gb_grid_create_unstructured(ug4gb_ctx *ctx, int elem_type, int num_vertices, const double *coords,
                                   int num_elements, const int *elems, const unsigned char *dirichlet_vertices,
                                   int num_dirichlet_edges, const int *dirichlet_edges, int num_dirichlet_faces,
                                   const int *dirichlet_faces, int nref, ug4gb_grid **out)
{
    if (!ctx || !coords || !elems || !out || num_vertices <= 0 || num_elements <= 0) return UG4GB_ERR_INVALID;
    if (num_dirichlet_edges < 0 || num_dirichlet_faces < 0) return UG4GB_ERR_INVALID;
    *out = nullptr;
    HostLevel L;
    const int rc = guarded(ctx, [&] {
        L.elem_type = elem_type;
        L.dim = dim_of(elem_type);
        L.k = corners_of(elem_type);
        L.nv = num_vertices;
        L.ne = num_elements;
        L.coords.assign(coords, coords + (size_t)num_vertices * L.dim);
        L.elems.assign(elems, elems + (size_t)num_elements * L.k);
        L.vdir.assign(num_vertices, 0);
        const bool whole = !dirichlet_vertices && num_dirichlet_edges == 0 && num_dirichlet_faces == 0;
        if (dirichlet_vertices) L.vdir.assign(dirichlet_vertices, dirichlet_vertices + num_vertices);
        for (int i = 0; i < num_dirichlet_edges; ++i) {
            const int a = dirichlet_edges[2 * i], b = dirichlet_edges[2 * i + 1];
            UG_REQUIRE(a >= 0 && a < num_vertices && b >= 0 && b < num_vertices && a != b, UG4GB_ERR_INVALID,
                       "grid: Dirichlet edge out of range");
            L.dir_edges.push_back(ekey(a, b));
            L.vdir[a] = L.vdir[b] = 1;
        }
        for (int i = 0; i < num_dirichlet_faces; ++i) {
            std::array<int, 4> f;
            for (int j = 0; j < 4; ++j) f[j] = dirichlet_faces[4 * i + j];
            for (int j = 0; j < 4; ++j) {
                UG_REQUIRE((j == 3 && f[j] == -1) || (f[j] >= 0 && f[j] < num_vertices), UG4GB_ERR_INVALID,
                           "grid: Dirichlet face corner out of range");
                if (f[j] >= 0) L.vdir[f[j]] = 1;
            }
            L.dir_faces.push_back(f);
        }
        check_level0(L);
        if (whole) {
            boundary_as_dirichlet(L);
            dedupe(L);
        }
    });
    if (rc != UG4GB_OK) return rc;
    return make_grid(ctx, std::move(L), nref, out);
}

int ug4gb_io_ugx_level(const char *filename, int nref, const char *dirichlet_subsets, int level, int *elem_type,
                       int *num_vertices, int *num_elements, double *coords, int *elems, unsigned char *dirichlet,
                       int *npar, int *par, char *err, int err_capacity)
{
    try {
        if (!filename || level < 0 || level > nref || nref > 10) fail("bad arguments");
        HostLevel L = ugx_level0(filename, dirichlet_subsets);
        for (int l = 0; l < level; ++l) {
            HostLevel next;
            refine(L, next);
            L = std::move(next);
        }
        if (elem_type) *elem_type = L.elem_type;
        if (num_vertices) *num_vertices = L.nv;
        if (num_elements) *num_elements = L.ne;
        if (coords) std::copy(L.coords.begin(), L.coords.end(), coords);
        if (elems) std::copy(L.elems.begin(), L.elems.end(), elems);
        if (dirichlet) std::copy(L.vdir.begin(), L.vdir.end(), dirichlet);
        if (npar && level > 0) std::copy(L.npar.begin(), L.npar.end(), npar);
        if (par && level > 0) std::copy(L.par.begin(), L.par.end(), par);
        return UG4GB_OK;
    } catch (const Error &e) {
        if (err && err_capacity > 0) snprintf(err, (size_t)err_capacity, "%s", e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc &) {
        if (err && err_capacity > 0) snprintf(err, (size_t)err_capacity, "out of host memory");
        return UG4GB_ERR_NOMEM;
    }
}

int ug4gb_grid_level_parents(const ug4gb_grid *g, int level, int *npar, int *par)
{
    if (!g || level < 1 || level >= (int)g->lev.size()) return UG4GB_ERR_INVALID;
    return guarded(g->ctx, [&] {
        const Level &L = g->lev[level];
        Ctx &c = g->ctx->c;
        if (npar) copy_out(c, npar, L.npar.p, sizeof(int) * (size_t)L.nv);
        if (par) copy_out(c, par, L.par.p, sizeof(int) * (size_t)L.nv * 8);
    });
}

int ug4gb_grid_is_structured(const ug4gb_grid *g)
{
    if (!g || g->lev.empty()) return UG4GB_ERR_INVALID;
    return g->lev[0].structured ? 1 : 0;
}

}  // extern "C"
