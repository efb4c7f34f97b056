// api_newton.cu -- NewtonSolver over the FV1 operator (host orchestration).
//
// Follows NewtonSolver::apply (lib_disc/operator/non_linear_operator/
// newton_solver/newton_impl.h:171-340) without Jacobian reuse or update
// hooks, optionally with StandardLineSearch:
//   prepare(u)          Dirichlet values into u (AssembledOperator::prepare ->
//                       DirichletBoundary::adjust_solution)
//   d = N(u)            assemble_defect (stationary or time-discrete)
//   start(|d|)
//   while not ended:    c = 0;  J = N'(u) (assemble_jacobian; with
//                       set_reassemble_J_freq(k > 0) only in steps 0, k, 2k, ...);
//                       linear solver (and its multigrid) init(J);
//                       apply(c, d) -- a failed linear solve ends Newton;
//                       u -= c;  prepare(u);  d = N(u);  update(|d|)
//                       (or the line search below in place of the update)
//   post()
// StandardLineSearch::search (line_search.h:186-400), from the defect norm
// |d_old| of the step's start and s = u:
//   for k = 1 .. max_steps:  u = u - lambda c;  prepare(u);  d = N(u);
//       rho_k = |d| / |d_old|;  accepted (and done, unless check_all) when
//       rho_k <= 1 - alpha |lambda|;  lambda *= reduce;
//       at k = max_steps: without accept_best the search (and Newton) fails;
//       else u = s - lambda_start reduce^best c for the first smallest rho,
//       d = N(u), failing when |d| > max_defect;
//       u = s before the next try.
// with StdConvCheck's rules (convergence_check_impl.h:130-172): ended when the
// defect is not a number, step >= max steps, defect < minimum defect or
// defect / initial defect < reduction; converged by the last two.
// Every step's work (assembly, multigrid set-up, Krylov solve, defect) runs
// in the library's kernels; the host reads one norm per Newton step.
#include <cmath>
#include <vector>

#include "gmg.cuh"

namespace ug4gb {
void disc_assemble(ug4gb_disc *d, int level, ug4gb_matrix *A, double *b, const TimeScale *ts);
void disc_defect(ug4gb_disc *d, int level, const double *u, double *dvec, const TimeScale *ts);
}  // namespace ug4gb

using namespace ug4gb;

struct ug4gb_newton {
    ug4gb_ctx *ctx = nullptr;
    ug4gb_disc *disc = nullptr;        // N(u) = stationary defect of disc, or
    ug4gb_timedisc *td = nullptr;      // the time-discrete defect of td
    ug4gb_solver *lin = nullptr;
    int maxit = 10;
    double min_def = 1e-50, rel_red = 1e-10;
    ug4gb_matrix *J = nullptr;
    ug4gb_vector *d = nullptr, *c = nullptr;
    int steps = 0;
    int j_freq = 0;                    // set_reassemble_J_freq (0: every step)
    int j_count = 0;                   // jacobian assemblies in the last apply
    double d0 = 0.0, dcur = 0.0;
    std::vector<int> lin_steps;
    std::vector<double> defects;
    // StandardLineSearch (off until set)
    bool ls_on = false;
    int ls_max = 10;
    double ls_start = 1.0, ls_reduce = 0.5, ls_alpha = 0.25, ls_max_defect = 1e10;
    bool ls_accept_best = false, ls_check_all = false;
    ug4gb_vector *s = nullptr;
    std::vector<int> ls_tries;          // per Newton step: tries evaluated
    std::vector<double> ls_lambda;      // per Newton step: the lambda of the accepted u
};

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
    } catch (const std::exception &e) {
        if (ctx) ctx->c.err = e.what();
        return UG4GB_ERR_INVALID;
    }
}

void check(ug4gb_ctx *ctx, int rc)
{
    if (rc != UG4GB_OK) throw Error{rc, ctx->c.err};
}

ug4gb_disc *op_disc(const ug4gb_newton *nw) { return nw->td ? nw->td->disc : nw->disc; }

void defect(ug4gb_newton *nw, const ug4gb_vector *u)
{
    ug4gb_disc *d = op_disc(nw);
    const int top = (int)d->g->lev.size() - 1;
    if (nw->td) {
        UG_REQUIRE(nw->td->prepared, UG4GB_ERR_STATE, "Newton: the time discretisation's prepare_step not called");
        const TimeScale ts = nw->td->defect_scale();
        disc_defect(d, top, u->d, nw->d->d, &ts);
    } else {
        disc_defect(d, top, u->d, nw->d->d, nullptr);
    }
}

void jacobian(ug4gb_newton *nw)
{
    ug4gb_disc *d = op_disc(nw);
    const int top = (int)d->g->lev.size() - 1;
    if (nw->td) {
        const TimeScale ts = nw->td->jacobian_scale();
        disc_assemble(d, top, nw->J, nullptr, &ts);
    } else {
        disc_assemble(d, top, nw->J, nullptr, nullptr);
    }
    UG_CUDA(cudaStreamSynchronize(nw->ctx->c.stream));
}

void prepare(ug4gb_newton *nw, ug4gb_vector *u)
{
    ug4gb_disc *d = op_disc(nw);
    launch_dirichlet_values(nw->ctx->c, d->g->lev.back(), u->d);
}

// is_valid_number (common/math/misc/math_util.h): 0, or a normal positive
// double (no NaN, no infinity, no subnormal)
bool valid(double v)
{
    if (v == 0.0) return true;
    return v >= 2.2250738585072014e-308 && v <= 1.7976931348623157e308 && v == v;
}

// StandardLineSearch::search; u = s - lambda c with d = N(u) on return,
// *norm = |d|.  Throws when the search fails.
void line_search(ug4gb_newton *nw, ug4gb_vector *u, double norm_old, double *norm)
{
    ug4gb_ctx *ctx = nw->ctx;
    check(ctx, ug4gb_vector_scale_add(nw->s, 1.0, u, 0.0, u));
    double lambda = nw->ls_start, nrm = 0.0, accepted = nw->ls_start;
    std::vector<double> rho;
    int tries = 0;
    for (int k = 1; k <= nw->ls_max; ++k) {
        check(ctx, ug4gb_vector_scale_add(u, 1.0, u, -lambda, nw->c));
        prepare(nw, u);
        defect(nw, u);
        check(ctx, ug4gb_vector_norm(nw->d, &nrm));
        tries = k;
        accepted = lambda;
        rho.push_back(nrm / norm_old);
        if (rho.back() <= 1.0 - nw->ls_alpha * std::fabs(lambda) && !nw->ls_check_all) break;
        lambda *= nw->ls_reduce;
        if (k == nw->ls_max) {
            if (!nw->ls_accept_best) {
                nw->ls_tries.push_back(tries);
                nw->ls_lambda.push_back(accepted);
                throw Error{UG4GB_ERR_NOT_CONVERGED, "NewtonSolver::apply: line search did not converge"};
            }
            size_t best = 0;
            for (size_t i = 1; i < rho.size(); ++i)
                if (rho[best] > rho[i]) best = i;
            accepted = nw->ls_start * std::pow(nw->ls_reduce, (double)best);
            check(ctx, ug4gb_vector_scale_add(u, 1.0, nw->s, -accepted, nw->c));
            prepare(nw, u);
            defect(nw, u);
            check(ctx, ug4gb_vector_norm(nw->d, &nrm));
            if (nrm > nw->ls_max_defect) {
                nw->ls_tries.push_back(tries);
                nw->ls_lambda.push_back(accepted);
                throw Error{UG4GB_ERR_NOT_CONVERGED, "StandardLineSearch::search: maximum defect-limit is reached"};
            }
            break;
        }
        check(ctx, ug4gb_vector_scale_add(u, 1.0, nw->s, 0.0, nw->s));
    }
    nw->ls_tries.push_back(tries);
    nw->ls_lambda.push_back(accepted);
    *norm = nrm;
}

bool ended(const ug4gb_newton *nw)
{
    if (!valid(nw->dcur)) return true;
    if (nw->steps >= nw->maxit) return true;
    if (nw->dcur < nw->min_def) return true;
    if (nw->dcur / nw->d0 < nw->rel_red) return true;
    return false;
}

}  // namespace

extern "C" {

int ug4gb_newton_create(ug4gb_ctx *ctx, ug4gb_newton **out)
{
    if (!ctx || !out) return UG4GB_ERR_INVALID;
    ug4gb_newton *nw = new ug4gb_newton;
    nw->ctx = ctx;
    ug4gb_ctx_retain(ctx);
    *out = nw;
    return UG4GB_OK;
}

int ug4gb_newton_set_linear_solver(ug4gb_newton *nw, ug4gb_solver *s)
{
    if (!nw || !s) return UG4GB_ERR_INVALID;
    nw->lin = s;
    return UG4GB_OK;
}

int ug4gb_newton_set_convergence_check(ug4gb_newton *nw, int max_steps, double min_defect, double reduction)
{
    if (!nw || max_steps < 0) return UG4GB_ERR_INVALID;
    nw->maxit = max_steps;
    nw->min_def = min_defect;
    nw->rel_red = reduction;
    return UG4GB_OK;
}

int ug4gb_newton_set_line_search(ug4gb_newton *nw, int max_steps, double lambda_start, double lambda_reduce,
                                 double suff_descent_factor, int accept_best, int check_all, double max_defect)
{
    if (!nw) return UG4GB_ERR_INVALID;
    if (max_steps < 1 || !(lambda_reduce > 0.0) || !std::isfinite(lambda_start) || !std::isfinite(max_defect)) {
        nw->ctx->c.err = "StandardLineSearch: max_steps >= 1, lambda_reduce > 0, finite lambda_start and max_defect";
        return UG4GB_ERR_INVALID;
    }
    nw->ls_on = true;
    nw->ls_max = max_steps;
    nw->ls_start = lambda_start;
    nw->ls_reduce = lambda_reduce;
    nw->ls_alpha = suff_descent_factor;
    nw->ls_accept_best = accept_best != 0;
    nw->ls_check_all = check_all != 0;
    nw->ls_max_defect = max_defect;
    return UG4GB_OK;
}

int ug4gb_newton_set_reassemble_J_freq(ug4gb_newton *nw, int freq)
{
    if (!nw || freq < 0) return UG4GB_ERR_INVALID;
    nw->j_freq = freq;
    return UG4GB_OK;
}

int ug4gb_newton_num_jacobian_assemblies(const ug4gb_newton *nw)
{
    return nw ? nw->j_count : UG4GB_ERR_INVALID;
}

int ug4gb_newton_clear_line_search(ug4gb_newton *nw)
{
    if (!nw) return UG4GB_ERR_INVALID;
    nw->ls_on = false;
    return UG4GB_OK;
}

int ug4gb_newton_get_line_search_history(const ug4gb_newton *nw, int *tries, double *lambdas, int capacity)
{
    if (!nw || capacity < 0) return UG4GB_ERR_INVALID;
    const int n = (int)nw->ls_tries.size();
    for (int i = 0; i < capacity && i < n; ++i) {
        if (tries) tries[i] = nw->ls_tries[i];
        if (lambdas) lambdas[i] = nw->ls_lambda[i];
    }
    return n;
}

int ug4gb_newton_init(ug4gb_newton *nw, ug4gb_disc *d, ug4gb_timedisc *td)
{
    if (!nw || (!d) == (!td)) return UG4GB_ERR_INVALID;
    nw->disc = d;
    nw->td = td;
    return UG4GB_OK;
}

int ug4gb_newton_prepare(ug4gb_newton *nw, ug4gb_vector *u)
{
    if (!nw || !u || (!nw->disc && !nw->td)) return UG4GB_ERR_INVALID;
    if (u->n != op_disc(nw)->g->lev.back().nv) return UG4GB_ERR_INVALID;
    return guarded(nw->ctx, [&] {
        prepare(nw, u);
        UG_CUDA(cudaStreamSynchronize(nw->ctx->c.stream));
    });
}

int ug4gb_newton_apply(ug4gb_newton *nw, ug4gb_vector *u)
{
    ug4gb::NvtxRange nvtx_("ug4gb:newton_apply");
    if (!nw || !u) return UG4GB_ERR_INVALID;
    if (!nw->lin || (!nw->disc && !nw->td)) {
        if (nw) nw->ctx->c.err = "NewtonSolver::apply: linear solver or operator not set";
        return UG4GB_ERR_STATE;
    }
    ug4gb_disc *dd = op_disc(nw);
    const int nv = dd->g->lev.back().nv;
    if (u->n != nv) return UG4GB_ERR_INVALID;
    bool converged = false;
    const int rc = guarded(nw->ctx, [&] {
        ug4gb_ctx *ctx = nw->ctx;
        if (!nw->J) check(ctx, ug4gb_matrix_create(ctx, &nw->J));
        if (!nw->d || nw->d->n != nv) {
            ug4gb_vector_destroy(nw->d);
            ug4gb_vector_destroy(nw->c);
            ug4gb_vector_destroy(nw->s);
            nw->d = nw->c = nw->s = nullptr;
            check(ctx, ug4gb_vector_create(ctx, nv, &nw->d));
            check(ctx, ug4gb_vector_create(ctx, nv, &nw->c));
            check(ctx, ug4gb_vector_create(ctx, nv, &nw->s));
        }
        nw->lin_steps.clear();
        nw->defects.clear();
        nw->ls_tries.clear();
        nw->ls_lambda.clear();
        nw->j_count = 0;
        prepare(nw, u);
        defect(nw, u);
        check(ctx, ug4gb_vector_norm(nw->d, &nw->d0));
        nw->dcur = nw->d0;
        nw->steps = 0;
        nw->defects.push_back(nw->d0);
        while (!ended(nw)) {
            check(ctx, ug4gb_vector_set(nw->c, 0.0));
            if (nw->j_freq == 0 || nw->steps % nw->j_freq == 0) {
                jacobian(nw);
                nw->j_count++;
            }
            if (nw->lin->pre) check(ctx, ug4gb_gmg_init(nw->lin->pre, nw->J));
            check(ctx, ug4gb_solver_init(nw->lin, nw->J));
            const int lrc = ug4gb_solver_apply(nw->lin, nw->c, nw->d);
            int ls = 0;
            ug4gb_solver_get_stats(nw->lin, &ls, nullptr, nullptr, nullptr);
            nw->lin_steps.push_back(ls);
            if (lrc != UG4GB_OK) {
                throw Error{lrc, std::string("NewtonSolver::apply: linear solver failed: ") + ctx->c.err};
            }
            double nd = 0.0;
            if (nw->ls_on) {
                line_search(nw, u, nw->dcur, &nd);
            } else {
                check(ctx, ug4gb_vector_scale_add(u, 1.0, u, -1.0, nw->c));
                prepare(nw, u);
                defect(nw, u);
                check(ctx, ug4gb_vector_norm(nw->d, &nd));
            }
            nw->dcur = nd;
            nw->steps++;
            nw->defects.push_back(nd);
        }
        converged = nw->dcur < nw->min_def || nw->dcur / nw->d0 < nw->rel_red;
    });
    if (rc != UG4GB_OK) return rc;
    if (!converged) {
        nw->ctx->c.err = "NewtonSolver::apply: not converged";
        return UG4GB_ERR_NOT_CONVERGED;
    }
    return UG4GB_OK;
}

int ug4gb_newton_get_stats(const ug4gb_newton *nw, int *steps, double *initial_defect, double *final_defect,
                           int *lin_steps, int capacity)
{
    if (!nw) return UG4GB_ERR_INVALID;
    if (steps) *steps = nw->steps;
    if (initial_defect) *initial_defect = nw->d0;
    if (final_defect) *final_defect = nw->dcur;
    if (lin_steps)
        for (int i = 0; i < capacity && i < (int)nw->lin_steps.size(); ++i) lin_steps[i] = nw->lin_steps[i];
    return UG4GB_OK;
}

int ug4gb_newton_get_history(const ug4gb_newton *nw, double *defects, int capacity)
{
    if (!nw || !defects) return UG4GB_ERR_INVALID;
    for (int i = 0; i < capacity && i < (int)nw->defects.size(); ++i) defects[i] = nw->defects[i];
    return (int)nw->defects.size();
}

void ug4gb_newton_destroy(ug4gb_newton *nw)
{
    if (!nw) return;
    ug4gb_ctx *ctx = nw->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    ug4gb_matrix_destroy(nw->J);
    ug4gb_vector_destroy(nw->d);
    ug4gb_vector_destroy(nw->c);
    ug4gb_vector_destroy(nw->s);
    delete nw;
    ug4gb_ctx_release(ctx);
}

}  // extern "C"
