// api_disc.cu -- C ABI: FV1 convection-diffusion discretisation (assembly,
// coefficients, Dirichlet rows) and the adjoint gradients.
#include <cstring>

#include "disc.cuh"
#include "gmg.cuh"

using namespace ug4gb;

namespace ug4gb {



// element coefficients of a level (cached until the coefficient changes)
const double *disc_coefficients(ug4gb_disc *d, int level)
{
    DiscImpl &D = d->d;
    Ctx &c = d->ctx->c;
    const auto &lev = d->g->lev;
    int nl = (int)lev.size();
    if ((int)D.Klev.size() != nl) {
        D.Klev.clear();
        D.Klev.resize(nl);
        D.Kvalid.assign(nl, false);
    }
    if (D.Kvalid[level]) return D.Klev[level].p;
    if (D.coef_kind == COEF_LOG_ELEMS) {
        // log K on every level from the top: children's mean, then exp
        std::vector<DevBuf<double>> logk(nl);
        logk[nl - 1].alloc(lev[nl - 1].ne);
        UG_CUDA(cudaMemcpyAsync(logk[nl - 1].p, D.m_top.p, D.m_top.bytes(), cudaMemcpyDeviceToDevice, c.stream));
        for (int l = nl - 2; l >= 0; --l) {
            logk[l].alloc(lev[l].ne);
            if (lev[l].structured) coarsen_log(c, lev[l + 1], lev[l], logk[l + 1].p, logk[l].p);
            else coarsen_log_children(c, lev[l + 1], lev[l], logk[l + 1].p, logk[l].p);
        }
        for (int l = 0; l < nl; ++l) {
            D.Klev[l].alloc(lev[l].ne);
            exp_elements(c, logk[l].p, lev[l].ne, D.Klev[l].p);
            D.Kvalid[l] = true;
        }
        UG_CUDA(cudaStreamSynchronize(c.stream));
        return D.Klev[level].p;
    }
    D.Klev[level].alloc(lev[level].ne);
    if (D.coef_kind == COEF_CONST) fill_double(c, D.Klev[level].p, lev[level].ne, D.K_const);
    else launch_coef_fourier(c, lev[level], D.kmodes, D.kk.p, D.kphase.p, D.kamp, D.kfactor, D.Klev[level].p);
    D.Kvalid[level] = true;
    return D.Klev[level].p;
}

// assemble the FV1 operator of `level` into A (and the rhs into b if given)
void disc_assemble(ug4gb_disc *d, int level, ug4gb_matrix *A, double *b, const TimeScale *ts)
{
    Ctx &c = d->ctx->c;
    const Level &L = d->g->lev[level];
    const double *K = disc_coefficients(d, level);
    const bool fresh = (A->pattern_grid != d->g->uid || A->pattern_level != level);
    if (fresh) {
        csr_from_elements(c, L, A->A);
        A->pattern_grid = d->g->uid;
        A->pattern_level = level;
    }
    A->op_valid = false;
    DiscImpl &D = d->d;
    bool top = (level == (int)d->g->lev.size() - 1);
    AsmArgs a;
    a.coords = L.coords.p;
    a.elems = L.elems.p;
    a.ne = L.ne;
    a.K = K;
    a.k_uniform = (D.coef_kind == COEF_CONST && c.row_assembly == 2) ? 1 : 0;
    a.k_value = D.K_const;
    a.f = (top && D.f_kind == 1) ? D.f_top.p : nullptr;
    a.f_seed = D.f_seed;
    a.use_seed = (top && D.f_kind == 2) ? 1 : 0;
    a.vmodes = D.upwind ? D.vmodes : 0;
    a.vk = D.vk.p;
    a.vc = D.vc.p;
    a.vphase = D.vphase.p;
    a.vscale = D.vscale;
    a.vel_version = D.vel_version;
    a.rowptr = A->A.rowptr.p;
    a.col = A->A.col.p;
    a.val = A->A.val.p;
    a.b = b;
    if (ts) {
        UG_REQUIRE(!b || (top && ts->u_old), UG4GB_ERR_INVALID,
                   "time-discrete right-hand side: top level with a previous solution only");
        a.inst = 1;
        a.sm0 = ts->sm0;
        a.sa0 = ts->sa0;
        a.sm1 = ts->sm1;
        a.sa1 = ts->sa1;
        a.u_old = ts->u_old;
    }
    // structured levels, stationary: row by row, every value written once
    if (c.row_assembly) {
        if (D.rows.size() < d->g->lev.size()) D.rows.resize(d->g->lev.size());
        if (launch_assemble_rows(c, L, a, D.rows[level])) return;
    }
    if (!fresh) UG_CUDA(cudaMemsetAsync(A->A.val.p, 0, sizeof(double) * (size_t)A->A.nnz, c.stream));
    if (b) UG_CUDA(cudaMemsetAsync(b, 0, sizeof(double) * (size_t)L.nv, c.stream));
    launch_assemble(c, L, a);
    launch_dirichlet(c, L, A->A, b);
}

// defect of u on `level` into dvec (stationary, or with ts the time-discrete
// defect of one step from ts->u_old)
void disc_defect(ug4gb_disc *d, int level, const double *u, double *dvec, const TimeScale *ts)
{
    Ctx &c = d->ctx->c;
    const Level &L = d->g->lev[level];
    const DiscImpl &D = d->d;
    const bool top = (level == (int)d->g->lev.size() - 1);
    UG_CUDA(cudaMemsetAsync(dvec, 0, sizeof(double) * (size_t)L.nv, c.stream));
    AsmArgs a;
    a.coords = L.coords.p;
    a.elems = L.elems.p;
    a.ne = L.ne;
    a.K = disc_coefficients(d, level);
    a.f = (top && D.f_kind == 1) ? D.f_top.p : nullptr;
    a.f_seed = D.f_seed;
    a.use_seed = (top && D.f_kind == 2) ? 1 : 0;
    a.vmodes = D.upwind ? D.vmodes : 0;
    a.vk = D.vk.p;
    a.vc = D.vc.p;
    a.vphase = D.vphase.p;
    a.vscale = D.vscale;
    a.vel_version = D.vel_version;
    a.rowptr = nullptr;
    a.col = nullptr;
    a.val = nullptr;
    a.b = nullptr;
    a.u = u;
    a.d = dvec;
    if (ts) {
        UG_REQUIRE(top && ts->u_old, UG4GB_ERR_INVALID, "time-discrete defect: top level with a previous solution");
        a.inst = 1;
        a.sm0 = ts->sm0;
        a.sa0 = ts->sa0;
        a.sm1 = ts->sm1;
        a.sa1 = ts->sa1;
        a.u_old = ts->u_old;
    }
    launch_defect(c, L, a);
}

}  // namespace ug4gb

template <class F>
static int guarded(ug4gb_ctx *ctx, F &&f)
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

static void invalidate(ug4gb_disc *d)
{
    d->d.Kvalid.assign(d->g->lev.size(), false);
}

extern "C" {

int ug4gb_disc_create(ug4gb_ctx *ctx, const ug4gb_grid *g, ug4gb_disc **out)
{
    if (!ctx || !g || !out) return UG4GB_ERR_INVALID;
    ug4gb_disc *d = new ug4gb_disc;
    d->ctx = ctx;
    d->g = g;
    invalidate(d);
    ug4gb_ctx_retain(ctx);
    *out = d;
    return UG4GB_OK;
}

int ug4gb_disc_set_diffusion_constant(ug4gb_disc *d, double K)
{
    if (!d) return UG4GB_ERR_INVALID;
    d->d.coef_kind = COEF_CONST;
    d->d.K_const = K;
    invalidate(d);
    return UG4GB_OK;
}

int ug4gb_disc_set_diffusion_fourier(ug4gb_disc *d, int nmodes, const double *k, const double *phase, double amp,
                                     double factor)
{
    if (!d || nmodes < 0 || (nmodes && (!k || !phase))) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        int dim = d->g->lev[0].dim;
        DiscImpl &D = d->d;
        D.coef_kind = COEF_FOURIER;
        D.kmodes = nmodes;
        D.kk.alloc((size_t)(nmodes > 0 ? nmodes : 1) * dim);
        D.kphase.alloc(nmodes > 0 ? nmodes : 1);
        copy_in(d->ctx->c, D.kk.p, k, sizeof(double) * (size_t)nmodes * dim);
        copy_in(d->ctx->c, D.kphase.p, phase, sizeof(double) * (size_t)nmodes);
        UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
        D.kamp = amp;
        D.kfactor = factor;
        invalidate(d);
    });
}

int ug4gb_disc_set_log_diffusion_elements(ug4gb_disc *d, const double *m_top)
{
    if (!d || !m_top) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        DiscImpl &D = d->d;
        int ne = d->g->lev.back().ne;
        D.coef_kind = COEF_LOG_ELEMS;
        D.m_top.alloc(ne);
        copy_in(d->ctx->c, D.m_top.p, m_top, sizeof(double) * (size_t)ne);
        // a device array is read in stream order (the caller keeps it
        // unchanged until the context's stream has passed this point)
        if (!is_device_ptr(m_top)) UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
        invalidate(d);
    });
}

int ug4gb_disc_set_velocity_fourier_curl(ug4gb_disc *d, int nmodes, const double *k, const double *cvec,
                                         const double *phase, double scale)
{
    if (!d || nmodes < 0 || (nmodes && (!k || !cvec || !phase))) return UG4GB_ERR_INVALID;
    if (d->g->lev[0].dim != 3 && nmodes > 0) {
        d->ctx->c.err = "velocity field: only 3D grids";
        return UG4GB_ERR_INVALID;
    }
    return guarded(d->ctx, [&] {
        DiscImpl &D = d->d;
        D.vmodes = nmodes;
        size_t m = nmodes > 0 ? nmodes : 1;
        D.vk.alloc(3 * m);
        D.vc.alloc(3 * m);
        D.vphase.alloc(m);
        copy_in(d->ctx->c, D.vk.p, k, sizeof(double) * 3 * (size_t)nmodes);
        copy_in(d->ctx->c, D.vc.p, cvec, sizeof(double) * 3 * (size_t)nmodes);
        copy_in(d->ctx->c, D.vphase.p, phase, sizeof(double) * (size_t)nmodes);
        UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
        D.vscale = scale;
        D.vel_version++;
    });
}

int ug4gb_disc_set_upwind(ug4gb_disc *d, int upwind)
{
    if (!d || (upwind != UG4GB_UPWIND_NONE && upwind != UG4GB_UPWIND_FULL)) return UG4GB_ERR_INVALID;
    d->d.upwind = upwind;
    return UG4GB_OK;
}

int ug4gb_disc_set_source_vertices(ug4gb_disc *d, const double *f)
{
    if (!d || !f) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        int nv = d->g->lev.back().nv;
        d->d.f_top.alloc(nv);
        copy_in(d->ctx->c, d->d.f_top.p, f, sizeof(double) * (size_t)nv);
        if (!is_device_ptr(f)) UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
        d->d.f_kind = 1;
    });
}

int ug4gb_disc_set_source_uniform(ug4gb_disc *d, uint64_t seed)
{
    if (!d) return UG4GB_ERR_INVALID;
    d->d.f_kind = 2;
    d->d.f_seed = seed;
    return UG4GB_OK;
}

int ug4gb_disc_assemble_linear(ug4gb_disc *d, int level, ug4gb_matrix *A, ug4gb_vector *b)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_assemble_linear");
    if (!d || !A || !b || level < 0 || level >= (int)d->g->lev.size()) return UG4GB_ERR_INVALID;
    if (b->n != d->g->lev[level].nv) {
        d->ctx->c.err = "assemble_linear: rhs size mismatch";
        return UG4GB_ERR_INVALID;
    }
    // queued on the context's stream (the matrix and rhs are device objects)
    return guarded(d->ctx, [&] { disc_assemble(d, level, A, b->d, nullptr); });
}

int ug4gb_disc_assemble_jacobian(ug4gb_disc *d, int level, ug4gb_matrix *A)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_assemble_jacobian");
    if (!d || !A || level < 0 || level >= (int)d->g->lev.size()) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] { disc_assemble(d, level, A, nullptr, nullptr); });
}

int ug4gb_disc_assemble_defect(ug4gb_disc *d, int level, const ug4gb_vector *u, ug4gb_vector *dvec)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_assemble_defect");
    if (!d || !u || !dvec || u == dvec || level < 0 || level >= (int)d->g->lev.size()) return UG4GB_ERR_INVALID;
    const int nv = d->g->lev[level].nv;
    if (u->n != nv || dvec->n != nv) {
        d->ctx->c.err = "assemble_defect: vector sizes != level vertices";
        return UG4GB_ERR_INVALID;
    }
    return guarded(d->ctx, [&] {
        disc_defect(d, level, u->d, dvec->d, nullptr);
        UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
    });
}

int ug4gb_disc_adjust_solution(ug4gb_disc *d, int level, ug4gb_vector *u)
{
    if (!d || !u || level < 0 || level >= (int)d->g->lev.size() || u->n != d->g->lev[level].nv)
        return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        launch_dirichlet_values(d->ctx->c, d->g->lev[level], u->d);
        UG_CUDA(cudaStreamSynchronize(d->ctx->c.stream));
    });
}

// ---- ThetaTimeStep ------------------------------------------------------
int ug4gb_timedisc_create(ug4gb_ctx *ctx, ug4gb_disc *d, ug4gb_timedisc **out)
{
    if (!ctx || !d || !out) return UG4GB_ERR_INVALID;
    ug4gb_timedisc *td = new ug4gb_timedisc;
    td->ctx = ctx;
    td->disc = d;
    ug4gb_ctx_retain(ctx);
    *out = td;
    return UG4GB_OK;
}

int ug4gb_timedisc_set_theta(ug4gb_timedisc *td, double theta)
{
    if (!td || !(theta >= 0.0 && theta <= 1.0)) return UG4GB_ERR_INVALID;
    td->theta = theta;
    return UG4GB_OK;
}

int ug4gb_timedisc_prepare_step(ug4gb_timedisc *td, const ug4gb_vector *u_old, double t_old, double dt)
{
    if (!td || !u_old || !(dt > 0.0)) return UG4GB_ERR_INVALID;
    const int nv = td->disc->g->lev.back().nv;
    if (u_old->n != nv) {
        td->ctx->c.err = "prepare_step: previous solution size != top level";
        return UG4GB_ERR_INVALID;
    }
    return guarded(td->ctx, [&] {
        Ctx &c = td->ctx->c;
        td->u_old.alloc(nv);
        UG_CUDA(cudaMemcpyAsync(td->u_old.p, u_old->d, sizeof(double) * (size_t)nv, cudaMemcpyDeviceToDevice,
                                c.stream));
        td->time = t_old;
        td->dt = dt;
        td->prepared = true;
    });
}

int ug4gb_timedisc_future_time(const ug4gb_timedisc *td, double *t)
{
    if (!td || !t) return UG4GB_ERR_INVALID;
    *t = td->time + td->dt;
    return UG4GB_OK;
}

int ug4gb_timedisc_assemble_linear(ug4gb_timedisc *td, int level, ug4gb_matrix *A, ug4gb_vector *b)
{
    ug4gb::NvtxRange nvtx_("ug4gb:timedisc_assemble_linear");
    if (!td || !A || !b) return UG4GB_ERR_INVALID;
    ug4gb_disc *d = td->disc;
    if (level != (int)d->g->lev.size() - 1 || b->n != d->g->lev[level].nv) {
        td->ctx->c.err = "time-discrete assemble_linear: top level, rhs of the level's size";
        return UG4GB_ERR_INVALID;
    }
    if (!td->prepared) {
        td->ctx->c.err = "time-discrete assemble_linear: prepare_step not called";
        return UG4GB_ERR_STATE;
    }
    return guarded(td->ctx, [&] {
        const TimeScale ts = td->scale();
        disc_assemble(d, level, A, b->d, &ts);
        UG_CUDA(cudaStreamSynchronize(td->ctx->c.stream));
    });
}

int ug4gb_timedisc_assemble_jacobian(ug4gb_timedisc *td, int level, ug4gb_matrix *A)
{
    ug4gb::NvtxRange nvtx_("ug4gb:timedisc_assemble_jacobian");
    if (!td || !A || level < 0 || level >= (int)td->disc->g->lev.size()) return UG4GB_ERR_INVALID;
    if (!td->prepared) {
        td->ctx->c.err = "time-discrete assemble_jacobian: prepare_step not called";
        return UG4GB_ERR_STATE;
    }
    return guarded(td->ctx, [&] {
        const TimeScale ts = td->jacobian_scale();
        disc_assemble(td->disc, level, A, nullptr, &ts);
        UG_CUDA(cudaStreamSynchronize(td->ctx->c.stream));
    });
}

int ug4gb_timedisc_assemble_defect(ug4gb_timedisc *td, int level, const ug4gb_vector *u, ug4gb_vector *dvec)
{
    ug4gb::NvtxRange nvtx_("ug4gb:timedisc_assemble_defect");
    if (!td || !u || !dvec || u == dvec) return UG4GB_ERR_INVALID;
    ug4gb_disc *d = td->disc;
    if (level != (int)d->g->lev.size() - 1 || u->n != d->g->lev[level].nv || dvec->n != u->n) {
        td->ctx->c.err = "time-discrete assemble_defect: top level, vectors of the level's size";
        return UG4GB_ERR_INVALID;
    }
    if (!td->prepared) {
        td->ctx->c.err = "time-discrete assemble_defect: prepare_step not called";
        return UG4GB_ERR_STATE;
    }
    return guarded(td->ctx, [&] {
        const TimeScale ts = td->defect_scale();
        disc_defect(d, level, u->d, dvec->d, &ts);
        UG_CUDA(cudaStreamSynchronize(td->ctx->c.stream));
    });
}

void ug4gb_timedisc_destroy(ug4gb_timedisc *td)
{
    if (!td) return;
    ug4gb_ctx *ctx = td->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete td;
    ug4gb_ctx_release(ctx);
}

int ug4gb_disc_adjoint_operator(ug4gb_disc *d, int level, const ug4gb_matrix *A, ug4gb_matrix *AT)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_adjoint_operator");
    if (!d || !A || !AT || level < 0 || level >= (int)d->g->lev.size()) return UG4GB_ERR_INVALID;
    if (A->A.nrows != d->g->lev[level].nv) return UG4GB_ERR_INVALID;
    if (A == AT) {
        // in place: the pattern is symmetric (checked once per pattern), the
        // values of each pair (i, j), (j, i) are swapped; no extra memory
        return guarded(d->ctx, [&] {
            Ctx &c = d->ctx->c;
            ug4gb_matrix *M = AT;
            const uint64_t key = M->pattern_key();
            if (!key || M->sym_key != key) {
                UG_REQUIRE(csr_pattern_symmetric(c, M->A), UG4GB_ERR_INVALID,
                           "adjoint operator in place: the operator's pattern is not symmetric");
                M->sym_key = key;
            }
            csr_transpose_symmetric_inplace(c, M->A);
            launch_dirichlet(c, d->g->lev[level], M->A, nullptr);
            M->op_valid = false;
        });
    }
    return guarded(d->ctx, [&] {
        Ctx &c = d->ctx->c;
        // the transposition of a level's element pattern is computed once;
        // later operators of the same pattern only move their values
        const uint64_t src = A->pattern_key();
        const uint64_t key = src ? (src | (1ULL << 63)) : 0;
        if (key && AT->tperm_key == src && AT->derived_key == key && AT->A.nnz == A->A.nnz) {
            transpose_values(c, A->A, AT->A, AT->tperm);
        } else {
            transpose_perm(c, A->A, AT->A, AT->tperm);
            AT->tperm_key = src;
        }
        launch_dirichlet(c, d->g->lev[level], AT->A, nullptr);
        AT->op_valid = false;
        AT->pattern_grid = 0;
        AT->pattern_level = -1;
        AT->derived_key = key;
    });
}

int ug4gb_disc_export_coefficients(ug4gb_disc *d, int level, double *K)
{
    if (!d || !K || level < 0 || level >= (int)d->g->lev.size()) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        const double *p = disc_coefficients(d, level);
        copy_out(d->ctx->c, K, p, sizeof(double) * (size_t)d->g->lev[level].ne);
    });
}

void ug4gb_disc_destroy(ug4gb_disc *d)
{
    if (!d) return;
    ug4gb_ctx *ctx = d->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete d;
    ug4gb_ctx_release(ctx);
}

int ug4gb_disc_grad_logk(ug4gb_disc *d, const ug4gb_vector *u, const ug4gb_vector *lam, double *grad)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_grad_logk");
    if (!d || !u || !lam || !grad) return UG4GB_ERR_INVALID;
    const Level &L = d->g->lev.back();
    if (u->n != L.nv || lam->n != L.nv) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        Ctx &c = d->ctx->c;
        const double *K = disc_coefficients(d, (int)d->g->lev.size() - 1);
        if (is_device_ptr(grad)) {
            // in stream order on the context's stream
            launch_grad_logk(c, L, K, u->d, lam->d, grad);
        } else {
            DevBuf<double> g;
            g.alloc(L.ne);
            launch_grad_logk(c, L, K, u->d, lam->d, g.p);
            copy_out(c, grad, g.p, g.bytes());
        }
    });
}

int ug4gb_disc_grad_source(ug4gb_disc *d, const ug4gb_vector *lam, double *grad)
{
    ug4gb::NvtxRange nvtx_("ug4gb:disc_grad_source");
    if (!d || !lam || !grad) return UG4GB_ERR_INVALID;
    const Level &L = d->g->lev.back();
    if (lam->n != L.nv) return UG4GB_ERR_INVALID;
    return guarded(d->ctx, [&] {
        Ctx &c = d->ctx->c;
        if (is_device_ptr(grad)) {
            launch_grad_source(c, L, lam->d, grad);
        } else {
            DevBuf<double> g;
            g.alloc(L.nv);
            launch_grad_source(c, L, lam->d, g.p);
            copy_out(c, grad, g.p, g.bytes());
        }
    });
}

}  // extern "C"
