// ref_fv1geom.cpp -- TEST INFRASTRUCTURE: runs ugcore's own FV1 element
// geometry (FV1Geometry, lib_disc/spatial_disc/disc_util/fv1_geom.cpp:259-464)
// and full-upwind convection shapes (ConvectionShapesFullUpwind::update,
// lib_disc/spatial_disc/disc_util/conv_shape.h:277-345), compiled from the
// reference sources where they lie (oracle/build_ref.sh), on elements read
// from stdin, and writes what they compute to stdout.  The fixtures made
// from its output (tests/golden/make_fv1geom_golden.py) pin the oracle's and
// the GPU's FV1 geometry and stencil to ugcore's code.
//
// Input:  elem_type (0 quad, 1 hex, 2 tet, 3 tri) num_elements num_modes scale
//         then num_modes lines "kx ky kz cx cy cz phase" of the velocity
//         field v(x) = scale * sum_m -sin(k_m . x + phase_m) c_m (3D; the
//         library's Fourier curl field), then per element: K and the corner
//         coordinates in reference order.
// Output per element: "S" SCV volumes; per SCVF "F from to normal ip
//         grad_0 .. grad_{k-1}"; per SCVF "U" the full-upwind shapes; "A" the
//         k x k element matrix of -div(K grad u) + div(v u) assembled from
//         them as the ConvectionDiffusion FV1 element disc does
//         (J(from, sh) += -(K grad_sh).n + conv(sh), J(to, sh) -= the same).
#include <cmath>
#include <cstdio>
#include <vector>

#include "lib_disc/spatial_disc/disc_util/conv_shape.h"

using namespace ug;

namespace {

struct Field {
    int nm = 0;
    double scale = 0.0;
    std::vector<double> k, c, ph;
    void eval(const double *x, int dim, double *v) const
    {
        for (int d = 0; d < dim; ++d) v[d] = 0.0;
        for (int m = 0; m < nm; ++m) {
            double a = ph[m];
            for (int d = 0; d < dim; ++d) a += k[3 * m + d] * x[d];
            const double s = -std::sin(a);
            for (int d = 0; d < dim; ++d) v[d] += s * c[3 * m + d];
        }
        for (int d = 0; d < dim; ++d) v[d] *= scale;
    }
};

template <typename TElem, int dim, int nc>
int run(int ne, const Field &F)
{
    FV1Geometry<TElem, dim> geo;
    ConvectionShapesFullUpwind<dim> up;
    for (int e = 0; e < ne; ++e) {
        double K;
        if (scanf("%lf", &K) != 1) return 1;
        MathVector<dim> c[nc];
        for (int i = 0; i < nc; ++i)
            for (int d = 0; d < dim; ++d)
                if (scanf("%lf", &c[i][d]) != 1) return 1;
        // update() skips the work when called twice for one element: a
        // distinct (never dereferenced) element address per element
        geo.update((GridObject *)(uintptr_t)(0x1000 + 64 * (uintptr_t)e), c, NULL);
        const size_t nf = geo.num_scvf();
        std::vector<MathVector<dim> > v(nf);
        for (size_t f = 0; f < nf; ++f) {
            double x[3], vv[3];
            for (int d = 0; d < dim; ++d) x[d] = geo.scvf(f).global_ip()[d];
            F.eval(x, dim, vv);
            for (int d = 0; d < dim; ++d) v[f][d] = vv[d];
        }
        if (!up.set_geometry_type(geo)) return 2;
        if (!up.update(&geo, &v[0], NULL, false)) return 2;
        printf("E %d\nS", e);
        for (size_t i = 0; i < geo.num_scv(); ++i) printf(" %.17g", geo.scv(i).volume());
        printf("\n");
        std::vector<double> A((size_t)nc * nc, 0.0);
        for (size_t f = 0; f < nf; ++f) {
            const auto &s = geo.scvf(f);
            printf("F %zu %zu", (size_t)s.from(), (size_t)s.to());
            for (int d = 0; d < dim; ++d) printf(" %.17g", s.normal()[d]);
            for (int d = 0; d < dim; ++d) printf(" %.17g", s.global_ip()[d]);
            for (int sh = 0; sh < nc; ++sh)
                for (int d = 0; d < dim; ++d) printf(" %.17g", s.global_grad(sh)[d]);
            printf("\nU");
            for (int sh = 0; sh < nc; ++sh) printf(" %.17g", up(f, sh));
            printf("\n");
            for (int sh = 0; sh < nc; ++sh) {
                double flux = 0.0;
                for (int d = 0; d < dim; ++d) flux += K * s.global_grad(sh)[d] * s.normal()[d];
                const double t = -flux + up(f, sh);
                A[s.from() * nc + sh] += t;
                A[s.to() * nc + sh] -= t;
            }
        }
        printf("A");
        for (double a : A) printf(" %.17g", a);
        printf("\n");
    }
    return 0;
}

}  // namespace

int main()
{
    int type, ne, nm;
    Field F;
    if (scanf("%d %d %d %lf", &type, &ne, &nm, &F.scale) != 4) return 1;
    F.nm = nm;
    F.k.resize(3 * (size_t)nm);
    F.c.resize(3 * (size_t)nm);
    F.ph.resize((size_t)nm);
    for (int m = 0; m < nm; ++m)
        if (scanf("%lf %lf %lf %lf %lf %lf %lf", &F.k[3 * m], &F.k[3 * m + 1], &F.k[3 * m + 2], &F.c[3 * m],
                  &F.c[3 * m + 1], &F.c[3 * m + 2], &F.ph[m]) != 7)
            return 1;
    switch (type) {
    case 0: return run<Quadrilateral, 2, 4>(ne, F);
    case 1: return run<Hexahedron, 3, 8>(ne, F);
    case 2: return run<Tetrahedron, 3, 4>(ne, F);
    case 3: return run<Triangle, 2, 3>(ne, F);
    }
    return 1;
}
