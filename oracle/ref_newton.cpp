/*
 * ref_newton.cpp -- runs ugcore's OWN NewtonSolver and StandardLineSearch on
 * the oracle's problems.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into
 * oracle/_ref/ref_newton from the reference sources in place (never copied).
 * It pins the restated Newton loop of the oracle (orc_prob_newton_ls,
 * oracle/ug4_oracle_api.c) against the reference classes:
 *   ug::NewtonSolver<CPUAlgebra>
 *       (lib_disc/operator/non_linear_operator/newton_solver/newton_impl.h:171-340),
 *   ug::StandardLineSearch (lib_disc/operator/non_linear_operator/line_search.h:115-400),
 *   ug::AssembledOperator / AssembledLinearOperator (prepare = adjust_solution,
 *       N(u) = assemble_defect, J = assemble_jacobian),
 *   ug::StdConvCheck (Newton and linear solver), ug::CG / ug::BiCGStab.
 * The discretisation (IAssemble) and the linear solver's multigrid come from
 * the restatement: the FV1 element discretisation is an external plugin and
 * the domain discretisation needs lib_grid, neither buildable here.  The
 * operator is the stationary one (theta < 0) or the theta step's from u_old;
 * the time scalings of that step are the restatement's.
 *
 * Usage: ref_newton <out.bin> elem mx my mz nref seed coef_kind diffusion
 *            theta dt maxit min_defect reduction ls_max ls_start ls_reduce
 *            ls_accept_best ls_check_all linear_rel_red
 * ls_max 0: no line search.  u starts from the seeded values
 * 0.1 * (2 u(seed + 7, i) - 1) (splitmix64 counter hash, as the oracle's
 * source), u_old = 0 for the theta step.
 * Output (little-endian binary): int steps, rc, nv, nrec, total linear
 * steps; nrec x double (the accepted lambda of every line search); nv x
 * double u; double initial (final / reduction) and final Newton defect.
 */
#include <cmath>
namespace boost { namespace math { using std::isnan; using std::isinf; } }

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "lib_algebra/cpu_algebra_types.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/linear_solver/cg.h"
#include "lib_algebra/operator/linear_solver/bicgstab.h"
#include "lib_algebra/operator/convergence_check.h"
#include "lib_disc/operator/non_linear_operator/newton_solver/newton.h"
#include "lib_disc/operator/non_linear_operator/line_search.h"

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
    double theta = -1.0, dt = 0.0;
    std::vector<double> u_old;
    std::vector<unsigned char> bnd;
    int nv = 0, top = 0;
};

/* the oracle's problem as ugcore's IAssemble: N(u) = the (theta-step)
   defect, J = its jacobian, adjust_solution = Dirichlet values 0 */
class OracleAssemble : public IAssemble<CPUAlgebra>
{
public:
    explicit OracleAssemble(Setup *s) : m_s(s), m_tuner(new AssemblingTuner<CPUAlgebra>) {}

    void assemble_jacobian(Mat &J, const Vec &u, const GridLevel &) override
    {
        orc_gmg G;
        std::vector<orc_crs> L((size_t)orc_prob_num_levels(m_s->P));
        std::memset(L.data(), 0, sizeof(orc_crs) * L.size());
        if (orc_prob_newton_gmg(m_s->P, m_s->theta, m_s->dt, &G, L.data())) UG_THROW("oracle jacobian failed");
        const orc_crs &A = L[m_s->top];
        J.resize_and_clear(A.n_rows, A.n_cols);
        for (int r = 0; r < A.n_rows; ++r)
            for (int a = A.rowptr[r]; a < A.rowptr[r + 1]; ++a) J(r, A.col[a]) = A.val[a];
        J.defragment();
        orc_prob_newton_gmg_free(m_s->P, &G, L.data());
        (void)u;
    }
    void assemble_defect(Vec &d, const Vec &u, const GridLevel &) override
    {
        std::vector<double> uu(m_s->nv), dd(m_s->nv);
        for (int i = 0; i < m_s->nv; ++i) uu[i] = u[i];
        if (orc_prob_defect(m_s->P, m_s->theta, m_s->dt, m_s->theta >= 0.0 ? m_s->u_old.data() : nullptr, uu.data(),
                            dd.data()))
            UG_THROW("oracle defect failed");
        for (int i = 0; i < m_s->nv; ++i) d[i] = dd[i];
    }
    void assemble_linear(Mat &, Vec &, const GridLevel &) override { UG_THROW("not used"); }
    void assemble_rhs(Vec &, const Vec &, const GridLevel &) override { UG_THROW("not used"); }
    void assemble_rhs(Vec &, const GridLevel &) override { UG_THROW("not used"); }
    void adjust_solution(Vec &u, const GridLevel &) override
    {
        for (int i = 0; i < m_s->nv; ++i)
            if (m_s->bnd[i]) u[i] = 0.0;
    }
    SmartPtr<AssemblingTuner<CPUAlgebra> > ass_tuner() override { return m_tuner; }
    ConstSmartPtr<AssemblingTuner<CPUAlgebra> > ass_tuner() const override { return m_tuner; }
    size_t num_constraints() const override { return 0; }
    SmartPtr<IConstraint<CPUAlgebra> > constraint(size_t) override { return SPNULL; }

private:
    Setup *m_s;
    SmartPtr<AssemblingTuner<CPUAlgebra> > m_tuner;
};

/* the oracle's GMG of the current jacobian as the linear solver's
   preconditioner (the restated multigrid; the Krylov method is ugcore's) */
class OracleGMG : public ILinearIterator<Vec>
{
public:
    explicit OracleGMG(Setup *s) : m_s(s) {}
    ~OracleGMG() override { release(); }
    const char *name() const override { return "OracleGMG"; }
    bool supports_parallel() const override { return false; }
    SmartPtr<ILinearIterator<Vec> > clone() override { return SPNULL; }
    bool init(SmartPtr<ILinearOperator<Vec> > J, const Vec &) override { return init(J); }
    bool init(SmartPtr<ILinearOperator<Vec> > J) override
    {
        release();
        m_J = J.template cast_dynamic<MatOp>();
        m_L.assign((size_t)orc_prob_num_levels(m_s->P), orc_crs());
        std::memset(m_L.data(), 0, sizeof(orc_crs) * m_L.size());
        m_ok = orc_prob_newton_gmg(m_s->P, m_s->theta, m_s->dt, &m_G, m_L.data()) == 0;
        return m_ok;
    }
    bool apply(Vec &c, const Vec &d) override
    {
        std::vector<double> cc(m_s->nv), dd(m_s->nv);
        for (int i = 0; i < m_s->nv; ++i) dd[i] = d[i];
        orc_gmg_apply(&m_G, cc.data(), dd.data());
        for (int i = 0; i < m_s->nv; ++i) c[i] = cc[i];
        return true;
    }
    bool apply_update_defect(Vec &c, Vec &d) override
    {
        if (!apply(c, d)) return false;
        m_J->apply_sub(d, c);
        return true;
    }

private:
    void release()
    {
        if (m_ok) orc_prob_newton_gmg_free(m_s->P, &m_G, m_L.data());
        m_ok = false;
    }
    Setup *m_s;
    SmartPtr<MatOp> m_J;
    orc_gmg m_G;
    std::vector<orc_crs> m_L;
    bool m_ok = false;
};

/* StandardLineSearch recording the accepted lambda of every search */
class RecordingLineSearch : public StandardLineSearch<Vec>
{
public:
    RecordingLineSearch(int maxSteps, number start, number reduce, bool acceptBest, bool checkAll)
        : StandardLineSearch<Vec>(maxSteps, start, reduce, acceptBest, checkAll)
    {}
    bool search(SmartPtr<IOperator<Vec> > spOp, Vec &u, Vec &p, Vec &d, number defect) override
    {
        Vec s;
        s.resize(u.size());
        s = u;
        const bool ok = StandardLineSearch<Vec>::search(spOp, u, p, d, defect);
        // the accepted lambda: u = s - lambda p at the largest |p|
        size_t im = 0;
        for (size_t i = 0; i < p.size(); ++i)
            if (std::fabs(p[i]) > std::fabs(p[im])) im = i;
        lambdas.push_back(p[im] != 0.0 ? (s[im] - u[im]) / p[im] : 0.0);
        return ok;
    }
    std::vector<double> lambdas;
};

double hash_unit(uint64_t seed, uint64_t i)
{
    uint64_t z = (seed ^ (i * 0xD1B54A32D192ED03ULL)) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 21) {
        std::fprintf(stderr, "usage: ref_newton out elem mx my mz nref seed coef_kind diffusion theta dt maxit "
                             "min_defect reduction ls_max ls_start ls_reduce ls_accept_best ls_check_all lin_red\n");
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
    p.diffusion = std::atof(argv[9]);
    p.peclet = 10.0;
    p.solver = 0;
    p.smoother = 0;
    p.damp = 0.6;
    p.nu1 = p.nu2 = 2;
    p.cycle = 1;
    p.maxit = 200;
    p.rel_red = std::atof(argv[20]);
    p.min_defect = 1e-300;
    p.damp_prol = p.damp_res = 1.0;
    p.post_smoother = -1;
    p.post_damp = 1.0;
    Setup s;
    s.theta = std::atof(argv[10]);
    s.dt = std::atof(argv[11]);
    const int maxit = std::atoi(argv[12]);
    const double min_def = std::atof(argv[13]), red = std::atof(argv[14]);
    const int ls_max = std::atoi(argv[15]);
    const double ls_start = std::atof(argv[16]), ls_reduce = std::atof(argv[17]);
    const bool ls_best = std::atoi(argv[18]) != 0, ls_all = std::atoi(argv[19]) != 0;

    s.P = orc_prob_create(&p, nullptr, nullptr);
    if (!s.P) return 3;
    s.top = orc_prob_num_levels(s.P) - 1;
    s.nv = orc_prob_level_nv(s.P, s.top);
    const int ne = orc_prob_level_ne(s.P, s.top);
    const int k = (p.elem_type == 1) ? 8 : 4;
    std::vector<int> elems((size_t)ne * k);
    std::vector<double> coords((size_t)s.nv * 3);
    s.bnd.assign(s.nv, 0);
    orc_prob_level_elems(s.P, s.top, elems.data(), coords.data(), s.bnd.data());
    s.u_old.assign(s.nv, 0.0);

    SmartPtr<OracleAssemble> ass = make_sp(new OracleAssemble(&s));
    SmartPtr<StdConvCheck<Vec> > lin_conv = make_sp(new StdConvCheck<Vec>(p.maxit, p.min_defect, p.rel_red, false));
    SmartPtr<CG<Vec> > cg = make_sp(new CG<Vec>());
    cg->set_preconditioner(make_sp(new OracleGMG(&s)));
    cg->set_convergence_check(lin_conv);
    NewtonSolver<CPUAlgebra> newton;
    newton.set_linear_solver(cg);
    SmartPtr<StdConvCheck<Vec> > conv = make_sp(new StdConvCheck<Vec>(maxit, min_def, red, false));
    newton.set_convergence_check(conv);
    SmartPtr<RecordingLineSearch> ls;
    if (ls_max > 0) {
        ls = make_sp(new RecordingLineSearch(ls_max, ls_start, ls_reduce, ls_best, ls_all));
        ls->set_verbose(false);
        newton.set_line_search(ls);
    }
    SmartPtr<AssembledOperator<CPUAlgebra> > op = make_sp(new AssembledOperator<CPUAlgebra>(ass));
    Vec u;
    u.resize(s.nv);
    for (int i = 0; i < s.nv; ++i) u[i] = 0.1 * (2.0 * hash_unit(p.seed + 7, (uint64_t)i) - 1.0);
    int rc = 0;
    std::vector<double> defects;
    try {
        newton.init(op);
        newton.prepare(u);
        rc = newton.apply(u) ? 0 : 1;
    } catch (UGError &e) {
        std::fprintf(stderr, "ugcore error: %s\n", e.get_msg().c_str());
        rc = 4;
    }
    const int steps = conv->step();
    std::vector<double> lam = ls.valid() ? ls->lambdas : std::vector<double>();
    const int nrec = (int)lam.size();
    FILE *f = std::fopen(argv[1], "wb");
    if (!f) return 5;
    const int hdr[5] = {steps, rc, s.nv, nrec, newton.total_linsolver_steps()};
    std::fwrite(hdr, sizeof(int), 5, f);
    std::fwrite(lam.data(), sizeof(double), (size_t)nrec, f);
    std::vector<double> uo(s.nv);
    for (int i = 0; i < s.nv; ++i) uo[i] = u[i];
    std::fwrite(uo.data(), sizeof(double), (size_t)s.nv, f);
    const double df[2] = {conv->defect() / conv->reduction(), conv->defect()};
    std::fwrite(df, sizeof(double), 2, f);
    std::fclose(f);
    orc_prob_free(s.P);
    return 0;
}
