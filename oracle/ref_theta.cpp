/*
 * ref_theta.cpp -- runs ugcore's OWN ThetaTimeStep on the oracle's problems.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into
 * oracle/_ref/ref_theta from the reference sources in place (never copied).
 * ugcore's ThetaTimeStep<CPUAlgebra> (lib_disc/time_disc/theta_time_step.h,
 * theta_time_step_impl.h: prepare_step, update_scaling, assemble_linear /
 * _jacobian / _defect through the time series of previous solutions) drives
 * a domain discretisation (IDomainDiscretization<CPUAlgebra>) whose
 * time-dependent assembly is the oracle's, called with exactly the time
 * scalings ThetaTimeStep passes (vScaleMass, vScaleStiff) and the previous
 * solution it pushes into the series.  The steps advance with ugcore's own
 * dense LU (lib_algebra/operator/linear_solver/lu.h).  This pins the
 * oracle's restated theta scalings and its use of the previous solution
 * against the reference; the spatial FV1 terms (mass and stiffness) stay
 * the restatement's.
 *
 * Usage: ref_theta <out.bin> elem mx my mz nref seed coef_kind theta dt nsteps
 * u starts from 0.1 * (2 u(seed + 7, i) - 1) (splitmix64 counter hash) with
 * the Dirichlet values set.
 * Output (little-endian binary): int nv, nnz, nsteps; then per step: the
 * scalings seen (4 doubles: sm0, sa0, sm1, sa1), u_old (nv), the step's
 * operator values (nnz, in the CRS order of the oracle's pattern), rhs (nv),
 * the defect of u_old + w (nv; w = 0.01 (2 u(seed + 11, i) - 1)), the
 * jacobian values (nnz).
 */
#include <cmath>
namespace boost { namespace math { using std::isnan; using std::isinf; } }

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "lib_algebra/cpu_algebra_types.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/linear_solver/lu.h"
#include "lib_disc/spatial_disc/domain_disc_interface.h"
#include "lib_disc/time_disc/theta_time_step.h"

extern "C" {
#include "ug4_oracle.h"
}

using namespace ug;
typedef CPUAlgebra::matrix_type Mat;
typedef CPUAlgebra::vector_type Vec;
typedef MatrixOperator<Mat, Vec> MatOp;

namespace {

struct Setup {
    orc_prob *P = nullptr;
    int nv = 0, top = 0;
    int64_t nnz = 0;
    std::vector<int> rowptr, col;
    std::vector<unsigned char> bnd;
    double scales[4] = {0, 0, 0, 0};   // the last scalings seen
};

void to_vec(const std::vector<double> &a, Vec &v)
{
    v.resize(a.size());
    for (size_t i = 0; i < a.size(); ++i) v[i] = a[i];
}

std::vector<double> from_vec(const Vec &v)
{
    std::vector<double> a(v.size());
    for (size_t i = 0; i < v.size(); ++i) a[i] = v[i];
    return a;
}

/* the oracle's discretisation as ugcore's IDomainDiscretization: only the
   time-dependent assembly a MultiStepTimeDiscretization calls is provided */
class OracleDomainDisc : public IDomainDiscretization<CPUAlgebra>
{
public:
    typedef IDomainDiscretization<CPUAlgebra>::error_vector_type error_vector_type;

    explicit OracleDomainDisc(Setup *s) : m_s(s), m_tuner(new AssemblingTuner<CPUAlgebra>) {}

    // ---- time-dependent assembly (the part under test)
    void assemble_jacobian(Mat &J, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const number s_a0,
                           const GridLevel &) override
    {
        // d/du of s_m0 M u + s_a0 (A u - f): the mass scaling of the current
        // time level is 1 for every one-step scheme of ugcore
        std::vector<double> b(m_s->nv), val(m_s->nnz), u_old = from_vec(*vSol->solution(vSol->size() - 1));
        if (orc_prob_scaled_system(m_s->P, 1.0, s_a0, 0.0, 0.0, u_old.data(), m_s->rowptr.data(), m_s->col.data(),
                                   val.data(), b.data()))
            UG_THROW("oracle jacobian failed");
        set_matrix(J, val);
    }
    void assemble_jacobian(Mat &J, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const number s_a0,
                           ConstSmartPtr<DoFDistribution>) override
    {
        assemble_jacobian(J, vSol, s_a0, GridLevel());
    }
    void assemble_defect(Vec &d, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                         const std::vector<number> &sa, const GridLevel &) override
    {
        check_two_levels(sm, sa, vSol);
        std::vector<double> u = from_vec(*vSol->solution(0)), u_old = from_vec(*vSol->solution(1)), dd(m_s->nv);
        if (orc_prob_scaled_defect(m_s->P, sm[0], sa[0], sm[1], sa[1], u_old.data(), u.data(), dd.data()))
            UG_THROW("oracle defect failed");
        to_vec(dd, d);
    }
    void assemble_defect(Vec &d, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                         const std::vector<number> &sa, ConstSmartPtr<DoFDistribution>) override
    {
        assemble_defect(d, vSol, sm, sa, GridLevel());
    }
    void assemble_linear(Mat &A, Vec &b, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                         const std::vector<number> &sa, const GridLevel &) override
    {
        check_two_levels(sm, sa, vSol);
        std::vector<double> u_old = from_vec(*vSol->solution(1)), bb(m_s->nv), val(m_s->nnz);
        if (orc_prob_scaled_system(m_s->P, sm[0], sa[0], sm[1], sa[1], u_old.data(), m_s->rowptr.data(),
                                   m_s->col.data(), val.data(), bb.data()))
            UG_THROW("oracle system failed");
        set_matrix(A, val);
        to_vec(bb, b);
    }
    void assemble_linear(Mat &A, Vec &b, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                         const std::vector<number> &sa, ConstSmartPtr<DoFDistribution>) override
    {
        assemble_linear(A, b, vSol, sm, sa, GridLevel());
    }
    void assemble_rhs(Vec &b, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                      const std::vector<number> &sa, const GridLevel &gl) override
    {
        Mat A;
        assemble_linear(A, b, vSol, sm, sa, gl);
    }
    void assemble_rhs(Vec &b, ConstSmartPtr<VectorTimeSeries<Vec> > vSol, const std::vector<number> &sm,
                      const std::vector<number> &sa, ConstSmartPtr<DoFDistribution>) override
    {
        assemble_rhs(b, vSol, sm, sa, GridLevel());
    }
    void prepare_timestep(ConstSmartPtr<VectorTimeSeries<Vec> >, number, ConstSmartPtr<DoFDistribution>) override {}
    void prepare_timestep(ConstSmartPtr<VectorTimeSeries<Vec> >, number, const GridLevel &) override {}
    void prepare_timestep_elem(ConstSmartPtr<VectorTimeSeries<Vec> >, ConstSmartPtr<DoFDistribution>) override {}
    void prepare_timestep_elem(ConstSmartPtr<VectorTimeSeries<Vec> >, const GridLevel &) override {}
    void finish_timestep(ConstSmartPtr<VectorTimeSeries<Vec> >, ConstSmartPtr<DoFDistribution>) override {}
    void finish_timestep(ConstSmartPtr<VectorTimeSeries<Vec> >, const GridLevel &) override {}
    void finish_timestep_elem(ConstSmartPtr<VectorTimeSeries<Vec> >, const GridLevel &) override {}
    void finish_timestep_elem(ConstSmartPtr<VectorTimeSeries<Vec> >, ConstSmartPtr<DoFDistribution>) override {}
    void adjust_solution(Vec &u, number, const GridLevel &gl) override { adjust_solution(u, gl); }
    void adjust_solution(Vec &u, number, ConstSmartPtr<DoFDistribution>) override { adjust_solution(u, GridLevel()); }
    void adjust_solution(Vec &u, const GridLevel &) override
    {
        for (int i = 0; i < m_s->nv; ++i)
            if (m_s->bnd[i]) u[i] = 0.0;
    }
    void adjust_solution(Vec &u, ConstSmartPtr<DoFDistribution>) override { adjust_solution(u, GridLevel()); }

    // ---- the stationary interface: not used by the time stepping
    void assemble_jacobian(Mat &, const Vec &, const GridLevel &) override { not_used(); }
    void assemble_jacobian(Mat &, const Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_defect(Vec &, const Vec &, const GridLevel &) override { not_used(); }
    void assemble_defect(Vec &, const Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_linear(Mat &, Vec &, const GridLevel &) override { not_used(); }
    void assemble_linear(Mat &, Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_rhs(Vec &, const Vec &, const GridLevel &) override { not_used(); }
    void assemble_rhs(Vec &, const Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_rhs(Vec &, const GridLevel &) override { not_used(); }
    void assemble_rhs(Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_mass_matrix(Mat &, const Vec &, const GridLevel &) override { not_used(); }
    void assemble_mass_matrix(Mat &, const Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    void assemble_stiffness_matrix(Mat &, const Vec &, const GridLevel &) override { not_used(); }
    void assemble_stiffness_matrix(Mat &, const Vec &, ConstSmartPtr<DoFDistribution>) override { not_used(); }
    SmartPtr<AssemblingTuner<CPUAlgebra> > ass_tuner() override { return m_tuner; }
    ConstSmartPtr<AssemblingTuner<CPUAlgebra> > ass_tuner() const override { return m_tuner; }
    size_t num_constraints() const override { return 0; }
    SmartPtr<IConstraint<CPUAlgebra> > constraint(size_t) override { return SPNULL; }
    void calc_error(const Vec &, const GridLevel &, error_vector_type * = NULL) override { not_used(); }
    void calc_error(const Vec &, ConstSmartPtr<DoFDistribution>, error_vector_type * = NULL) override { not_used(); }
    void calc_error(ConstSmartPtr<VectorTimeSeries<Vec> >, ConstSmartPtr<DoFDistribution>,
                    const std::vector<number> &, const std::vector<number> &, error_vector_type *) override
    {
        not_used();
    }
    void calc_error(ConstSmartPtr<VectorTimeSeries<Vec> >, const std::vector<number> &, const std::vector<number> &,
                    const GridLevel &, error_vector_type *) override
    {
        not_used();
    }
    void invalidate_error() override {}
    bool is_error_valid() override { return false; }

private:
    [[noreturn]] static void not_used() { UG_THROW("OracleDomainDisc: not used by the time stepping"); }
    void check_two_levels(const std::vector<number> &sm, const std::vector<number> &sa,
                          ConstSmartPtr<VectorTimeSeries<Vec> > vSol)
    {
        UG_COND_THROW(sm.size() != 2 || sa.size() != 2 || vSol->size() != 2, "one previous time level expected");
        m_s->scales[0] = sm[0];
        m_s->scales[1] = sa[0];
        m_s->scales[2] = sm[1];
        m_s->scales[3] = sa[1];
    }
    void set_matrix(Mat &A, const std::vector<double> &val)
    {
        A.resize_and_clear(m_s->nv, m_s->nv);
        for (int r = 0; r < m_s->nv; ++r)
            for (int a = m_s->rowptr[r]; a < m_s->rowptr[r + 1]; ++a) A(r, m_s->col[a]) = val[a];
        A.defragment();
    }
    Setup *m_s;
    SmartPtr<AssemblingTuner<CPUAlgebra> > m_tuner;
};

double hash_unit(uint64_t seed, uint64_t i)
{
    uint64_t z = (seed ^ (i * 0xD1B54A32D192ED03ULL)) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* the values of A in the CRS order of the given pattern */
std::vector<double> values_in_pattern(const Mat &A, const Setup &s)
{
    std::vector<double> v(s.nnz, 0.0);
    for (int r = 0; r < s.nv; ++r)
        for (int a = s.rowptr[r]; a < s.rowptr[r + 1]; ++a) v[a] = A(r, s.col[a]);
    return v;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 12) {
        std::fprintf(stderr, "usage: ref_theta out elem mx my mz nref seed coef_kind theta dt nsteps\n");
        return 2;
    }
    orc_params p;
    std::memset(&p, 0, sizeof(p));
    p.elem_type = std::atoi(argv[2]);
    p.mx = std::atoi(argv[3]);
    p.my = std::atoi(argv[4]);
    p.mz = std::atoi(argv[5]);
    p.nref = std::atoi(argv[6]);
    p.seed = std::strtoull(argv[7], nullptr, 10);
    p.coef_kind = std::atoi(argv[8]);
    p.coef_modes = 64;
    p.coef_kmax = 8.0;
    p.vel_modes = 16;
    p.vel_kmax = 2.0;
    p.diffusion = 1.0;
    p.peclet = 10.0;
    p.damp = 0.6;
    p.nu1 = p.nu2 = 2;
    p.cycle = 1;
    p.maxit = 200;
    p.rel_red = 1e-10;
    p.min_defect = 1e-300;
    p.damp_prol = p.damp_res = 1.0;
    p.post_smoother = -1;
    p.post_damp = 1.0;
    const double theta = std::atof(argv[9]), dt = std::atof(argv[10]);
    const int nsteps = std::atoi(argv[11]);

    Setup s;
    s.P = orc_prob_create(&p, nullptr, nullptr);
    if (!s.P) return 3;
    s.top = orc_prob_num_levels(s.P) - 1;
    s.nv = orc_prob_level_nv(s.P, s.top);
    s.nnz = orc_prob_level_nnz(s.P, s.top);
    s.rowptr.resize(s.nv + 1);
    s.col.resize(s.nnz);
    {
        std::vector<double> val(s.nnz);
        orc_prob_level_matrix(s.P, s.top, s.rowptr.data(), s.col.data(), val.data());
        const int ne = orc_prob_level_ne(s.P, s.top);
        const int k = (p.elem_type == 1) ? 8 : (p.elem_type == 3 ? 3 : 4);
        std::vector<int> elems((size_t)ne * k);
        std::vector<double> coords((size_t)s.nv * 3);
        s.bnd.assign(s.nv, 0);
        orc_prob_level_elems(s.P, s.top, elems.data(), coords.data(), s.bnd.data());
    }
    SmartPtr<OracleDomainDisc> dd = make_sp(new OracleDomainDisc(&s));
    ThetaTimeStep<CPUAlgebra> td(dd, theta);

    std::vector<double> u0(s.nv);
    for (int i = 0; i < s.nv; ++i) u0[i] = s.bnd[i] ? 0.0 : 0.1 * (2.0 * hash_unit(p.seed + 7, (uint64_t)i) - 1.0);
    SmartPtr<Vec> u = make_sp(new Vec());
    to_vec(u0, *u);
    SmartPtr<VectorTimeSeries<Vec> > series = make_sp(new VectorTimeSeries<Vec>());
    series->push(u->clone(), 0.0);

    FILE *f = std::fopen(argv[1], "wb");
    if (!f) return 5;
    const int hdr[3] = {s.nv, (int)s.nnz, nsteps};
    std::fwrite(hdr, sizeof(int), 3, f);
    LU<CPUAlgebra> lu;
    double t = 0.0;
    try {
        for (int step = 0; step < nsteps; ++step) {
            td.prepare_step(series, dt);
            SmartPtr<MatOp> A = make_sp(new MatOp());
            Vec b;
            td.assemble_linear(*A, b, GridLevel());
            const double sc[4] = {s.scales[0], s.scales[1], s.scales[2], s.scales[3]};
            const std::vector<double> uold = from_vec(*series->latest());
            // defect and jacobian at u_old + w
            Vec w;
            w.resize(s.nv);
            for (int i = 0; i < s.nv; ++i) w[i] = uold[i] + 0.01 * (2.0 * hash_unit(p.seed + 11, (uint64_t)i) - 1.0);
            Vec d;
            d.resize(s.nv);
            td.assemble_defect(d, w, GridLevel());
            Mat J;
            td.assemble_jacobian(J, w, GridLevel());
            std::fwrite(sc, sizeof(double), 4, f);
            std::fwrite(uold.data(), sizeof(double), (size_t)s.nv, f);
            const std::vector<double> av = values_in_pattern(*A, s), bv = from_vec(b), dv = from_vec(d),
                                      jv = values_in_pattern(J, s);
            std::fwrite(av.data(), sizeof(double), (size_t)s.nnz, f);
            std::fwrite(bv.data(), sizeof(double), (size_t)s.nv, f);
            std::fwrite(dv.data(), sizeof(double), (size_t)s.nv, f);
            std::fwrite(jv.data(), sizeof(double), (size_t)s.nnz, f);
            // advance with ugcore's dense LU
            lu.init(A);
            SmartPtr<Vec> un = make_sp(new Vec());
            un->resize(s.nv);
            un->set(0.0);
            lu.apply(*un, b);
            t = td.future_time();
            series->push_discard_oldest(un, t);
        }
    } catch (UGError &e) {
        std::fprintf(stderr, "ugcore error: %s\n", e.get_msg().c_str());
        std::fclose(f);
        return 4;
    }
    std::fclose(f);
    orc_prob_free(s.P);
    return 0;
}
