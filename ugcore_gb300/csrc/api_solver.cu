// api_solver.cu -- CG / BiCGStab drivers with StdConvCheck on the device.
//
// A solve is captured once as a CUDA graph: the prologue (r = b - A x, the
// first defect and, for CG, the first step), a kernel that tests the
// convergence flag, and a conditional WHILE node (body: one Krylov
// iteration, preconditioner cycle included, and the same test); it is
// launched once per solve.  All scalars (alpha, beta, rho, omega, defects)
// stay in device memory, the device-side convergence check ends the loop,
// and every kernel returns at once when the convergence flag is set.  The
// host waits once per solve, for the scalars and the defect history
// together.  The iteration count, defect
// history and stopping rule are those of the reference loop
// (lib_algebra/operator/linear_solver/cg.h:103-230,
//  lib_algebra/operator/linear_solver/bicgstab.h:112-400,
//  lib_algebra/operator/convergence_check_impl.h:85-172).
#include <cstring>

#include "gmg.cuh"

using namespace ug4gb;

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

// the device buffers of an operator's solve format
static uint64_t op_signature(const OpMat<double> &M)
{
    uint64_t h = 1469598103934665603ULL;
    auto mix = [&](uint64_t v) {
        h ^= v;
        h *= 1099511628211ULL;
    };
    mix((uint64_t)M.kind);
    mix((uint64_t)M.nrows);
    mix((uint64_t)(uintptr_t)M.dia.val.p);
    mix((uint64_t)M.dia.S);
    mix((uint64_t)(uintptr_t)M.sell.val.p);
    mix((uint64_t)(uintptr_t)M.sell.col.p);
    mix((uint64_t)(uintptr_t)M.sell.sptr.p);
    mix((uint64_t)(uintptr_t)M.sell.swidth.p);
    return h;
}

static void drop_graph(ug4gb_solver *s)
{
    if (s->iter_graph) cudaGraphExecDestroy(s->iter_graph);
    s->iter_graph = nullptr;
    s->graph_x = nullptr;
}

static void free_pinned(ug4gb_solver *s)
{
    if (s->pinned) cudaFreeHost(s->pinned);
    s->pinned = nullptr;
    s->pinned_bytes = 0;
}

namespace {

// RedArgs for the solver's scalar block (its own counter slot)
RedArgs red_of(ug4gb_solver *s)
{
    Ctx &c = s->ctx->c;
    return RedArgs{c.red_partials.p, c.red_counter.p, s->ks.p};
}

// z = M d (or z = d without preconditioner), always FP64; rho fused when possible
const double *precond(ug4gb_solver *s, const double *d, const double *r_rho, int rho_kind)
{
    Ctx &c = s->ctx->c;
    RedArgs red = red_of(s);
    // Inside the CG loop body the preconditioner never runs after the check
    // has ended (the loop condition is tested after cg_update), so only
    // BiCGStab, whose check runs between its two half steps, needs the
    // kernels to test the done flag.
    const int *skip = s->kind == UG4GB_SOLVER_BICGSTAB ? &s->ks.p->done : nullptr;
    if (!s->pre) {
        if (r_rho) rho_dot<double>(c, s->n, d, r_rho, rho_kind, red);
        return d;
    }
    bool fused = false;
    // CG: d is r, whose FP32 copy krylov_start / cg_update already wrote
    const bool ready = s->kind == UG4GB_SOLVER_CG && s->pre->impl->top_defect_buffer() != nullptr;
    const double *z = s->pre->impl->apply(c, d, skip, r_rho, &red, rho_kind, fused, ready);
    if (r_rho && !fused) rho_dot<double>(c, s->n, z, r_rho, rho_kind, red);
    return z;
}

void cg_iteration(ug4gb_solver *s, double *x, double *r, bool first)
{
    Ctx &c = s->ctx->c;
    RedArgs red = red_of(s);
    const double *z = precond(s, r, r, first ? 0 : 1);
    c.prof_tag = "K";
    cg_spmv_dot_t<double>(c, s->A->op, z, s->p.p, s->q.p, first ? 1 : 0, red);
    cg_update(c, s->n, x, r, s->p.p, s->q.p, red, s->pre ? s->pre->impl->top_defect_buffer() : nullptr);
}

void bicg_iteration(ug4gb_solver *s, double *x, double *r)
{
    Ctx &c = s->ctx->c;
    RedArgs red = red_of(s);
    const int n = s->n;
    c.prof_tag = "K";
    bicg_restart(c, n, r, s->r0.p, s->p.p, s->v.p, red);
    bicg_rho(c, n, s->r0.p, r, red);
    bicg_p(c, n, r, s->p.p, s->v.p, red);
    const double *q = precond(s, s->p.p, nullptr, 0);
    c.prof_tag = "K";
    bicg_spmv_dot_t<double>(c, s->A->op, q, s->v.p, s->r0.p, red);
    bicg_x_s<double>(c, n, x, q, r, s->v.p, s->s.p, red);
    bicg_s_to_r(c, n, s->s.p, r, red);
    q = precond(s, s->s.p, nullptr, 0);
    c.prof_tag = "K";
    bicg_spmv_2dot_t<double>(c, s->A->op, q, s->t.p, s->s.p, red);
    bicg_x_r<double>(c, n, x, q, s->s.p, s->t.p, r, red);
}

// the entry test after the prologue and the last node of the loop body:
// (keep) iterating while the check has not ended
__global__ void k_loop_cond(cudaGraphConditionalHandle h, const KScal *ks)
{
    PDL_ENTRY();
    cudaGraphSetConditional(h, ks->done ? 0u : 1u);
}

void iteration(ug4gb_solver *s, double *x, double *r)
{
    if (s->kind == UG4GB_SOLVER_CG) cg_iteration(s, x, r, false);
    else bicg_iteration(s, x, r);
}

// r = b - A x starts the check; CG also does its first step
void prologue(ug4gb_solver *s, double *x, double *r)
{
    Ctx &c = s->ctx->c;
    RedArgs red = red_of(s);
    c.prof_tag = "K";
    krylov_start(c, s->A->op, x, r, red,
                 s->kind == UG4GB_SOLVER_CG && s->pre ? s->pre->impl->top_defect_buffer() : nullptr);
    if (s->kind == UG4GB_SOLVER_CG) cg_iteration(s, x, r, true);
}

// The whole solve as one graph: the prologue and k_loop_cond (captured), then
// a conditional WHILE node whose body is one Krylov iteration (multigrid
// cycle included) followed by k_loop_cond.  The loop ends when the
// device-side StdConvCheck (or a breakdown) sets done, at the latest after
// max_steps iterations; a solve that ends in the prologue skips it.
void build_loop_graph(ug4gb_solver *s, double *x, double *r)
{
    Ctx &c = s->ctx->c;
    cudaGraph_t g;
    UG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaGraphExec_t exec = nullptr;
    int64_t before = c.launches;
    try {
        UG_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
        UG_CUDA(cudaStreamBeginCaptureToGraph(c.stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
            prologue(s, x, r);
            UG_LAUNCH_PDL(c, k_loop_cond, 1, 1, 0, h, (const KScal *)s->ks.p);
        } catch (...) {
            cudaGraph_t tmp;
            cudaStreamEndCapture(c.stream, &tmp);
            throw;
        }
        {
            cudaGraph_t tmp;
            UG_CUDA(cudaStreamEndCapture(c.stream, &tmp));
        }
        s->prologue_kernels = c.launches - before;
        // the loop follows the captured chain's last node (the entry test)
        size_t nn = 0;
        UG_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
        std::vector<cudaGraphNode_t> nodes(nn);
        UG_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
        cudaGraphNode_t leaf = nullptr;
        int leaves = 0;
        for (cudaGraphNode_t nd : nodes) {
            size_t nout = 0;
            UG_CUDA(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &nout));
            if (nout == 0) {
                leaf = nd;
                ++leaves;
            }
        }
        UG_REQUIRE(leaves == 1, UG4GB_ERR_CUDA, "solver graph: the captured prologue is not one chain");
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        UG_CUDA(cudaGraphAddNode(&node, g, &leaf, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        const int64_t body_start = c.launches;
        UG_CUDA(cudaStreamBeginCaptureToGraph(c.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        try {
            iteration(s, x, r);
            UG_LAUNCH_PDL(c, k_loop_cond, 1, 1, 0, h, (const KScal *)s->ks.p);
        } catch (...) {
            cudaGraph_t tmp;
            cudaStreamEndCapture(c.stream, &tmp);
            throw;
        }
        cudaGraph_t tmp;
        UG_CUDA(cudaStreamEndCapture(c.stream, &tmp));
        s->iter_kernels = c.launches - body_start;
        UG_CUDA(cudaGraphInstantiate(&exec, g, 0));
    } catch (...) {
        c.launches = before;
        cudaGraphDestroy(g);
        throw;
    }
    cudaGraphDestroy(g);
    c.launches = before;
    s->iter_graph = exec;
}

void read_flags(ug4gb_solver *s, int *done)
{
    Ctx &c = s->ctx->c;
    UG_CUDA(cudaMemcpyAsync(c.host_pinned, &s->ks.p->done, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    *done = *(int *)c.host_pinned;
}

void run(ug4gb_solver *s, double *x, double *r)
{
    Ctx &c = s->ctx->c;
    UG_REQUIRE(s->A, UG4GB_ERR_STATE, "solver: init() not called");
    UG_REQUIRE(!s->pre || s->pre->impl, UG4GB_ERR_STATE, "solver: preconditioner not initialised");
    UG_REQUIRE(!s->pre || s->pre->n_top == s->n, UG4GB_ERR_INVALID, "solver: preconditioner size mismatch");
    // device scalars + history
    KScal h{};
    h.maxit = s->maxit;
    h.min_def = s->min_def;
    h.rel_red = s->rel_red;
    h.num_restarts = s->num_restarts;
    h.min_ortho = s->min_ortho;
    h.hist_cap = s->maxit + 2;
    s->hist.alloc(h.hist_cap);
    h.hist = s->hist.p;
    UG_CUDA(cudaMemcpyAsync(s->ks.p, &h, sizeof(KScal), cudaMemcpyHostToDevice, c.stream));
    if (c.profiling) {
        // profiled run: direct launches, each one timed with events
        prologue(s, x, r);
        int done = 0;
        read_flags(s, &done);
        while (!done) {
            iteration(s, x, r);
            read_flags(s, &done);
        }
    } else {
        int pre_gen = s->pre ? s->pre->gen : -1;
        if (!s->iter_graph || s->graph_x != x || s->graph_r != r || s->graph_pre_gen != pre_gen) {
            drop_graph(s);
            try {
                build_loop_graph(s, x, r);
            } catch (const Error &e) {
                // a driver that rejects programmatic edges inside a conditional
                // body: rebuild the loop with plain stream-ordered launches
                if (e.code != UG4GB_ERR_CUDA || !c.pdl) throw;
                (void)cudaGetLastError();
                c.pdl = false;
                build_loop_graph(s, x, r);
            }
            s->graph_x = x;
            s->graph_r = r;
            s->graph_pre_gen = pre_gen;
        }
        UG_CUDA(cudaGraphLaunch(s->iter_graph, c.stream));
    }
    // the scalars and the whole history buffer in one wait
    const size_t hist_off = (sizeof(KScal) + 15) / 16 * 16;
    const size_t need = hist_off + sizeof(double) * (size_t)h.hist_cap;
    if (s->pinned_bytes < need) {
        UG_CUDA(cudaStreamSynchronize(c.stream));
        free_pinned(s);
        UG_CUDA(cudaMallocHost(&s->pinned, need));
        s->pinned_bytes = need;
    }
    UG_CUDA(cudaMemcpyAsync(s->pinned, s->ks.p, sizeof(KScal), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaMemcpyAsync((char *)s->pinned + hist_off, s->hist.p, sizeof(double) * (size_t)h.hist_cap,
                            cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    std::memcpy(&s->host_ks, s->pinned, sizeof(KScal));
    if (s->pre && s->pre->impl) s->pre->impl->check_base();
    check_device_error(c);
    int steps_before = s->kind == UG4GB_SOLVER_CG ? 1 : 0;
    if (!c.profiling && s->iter_graph) {
        // the graph's prologue, and its loop body once per CG step / per
        // BiCGStab pair of half steps
        c.launches += s->prologue_kernels;
        if (s->host_ks.step > steps_before) {
            int64_t runs = s->kind == UG4GB_SOLVER_CG ? s->host_ks.step - steps_before : (s->host_ks.step + 1) / 2;
            c.launches += runs * s->iter_kernels;
        }
    }
    int nh = s->host_ks.step + 1 < h.hist_cap ? s->host_ks.step + 1 : h.hist_cap;
    s->host_hist.resize(nh);
    std::memcpy(s->host_hist.data(), (const char *)s->pinned + hist_off, sizeof(double) * nh);
    const KScal &k = s->host_ks;
    bool converged = (k.dcur < k.min_def) || (k.dcur / k.d0 < k.rel_red);
    if (k.fail) {
        s->last_rc = UG4GB_ERR_BREAKDOWN;
        throw Error{UG4GB_ERR_BREAKDOWN, "Krylov solver breakdown (zero denominator)"};
    }
    if (!converged) {
        s->last_rc = UG4GB_ERR_NOT_CONVERGED;
        throw Error{UG4GB_ERR_NOT_CONVERGED, "Krylov solver: maximum number of steps reached without convergence"};
    }
    s->last_rc = UG4GB_OK;
}

}  // namespace

extern "C" {

int ug4gb_solver_create(ug4gb_ctx *ctx, int kind, ug4gb_solver **out)
{
    if (!ctx || !out || (kind != UG4GB_SOLVER_CG && kind != UG4GB_SOLVER_BICGSTAB)) return UG4GB_ERR_INVALID;
    ug4gb_solver *s = new ug4gb_solver;
    s->ctx = ctx;
    s->kind = kind;
    int rc = guarded(ctx, [&] { s->ks.alloc(1); });
    if (rc != UG4GB_OK) {
        delete s;
        return rc;
    }
    ug4gb_ctx_retain(ctx);
    *out = s;
    return UG4GB_OK;
}

int ug4gb_solver_set_preconditioner(ug4gb_solver *s, ug4gb_gmg *m)
{
    if (!s) return UG4GB_ERR_INVALID;
    drop_graph(s);
    s->pre = m;
    return UG4GB_OK;
}

int ug4gb_solver_set_convergence_check(ug4gb_solver *s, int maxit, double min_def, double rel_red)
{
    if (!s || maxit < 0) return UG4GB_ERR_INVALID;
    drop_graph(s);
    s->maxit = maxit;
    s->min_def = min_def;
    s->rel_red = rel_red;
    return UG4GB_OK;
}

int ug4gb_solver_set_restart(ug4gb_solver *s, int num_restarts)
{
    if (!s || num_restarts < 0 || s->kind != UG4GB_SOLVER_BICGSTAB) return UG4GB_ERR_INVALID;
    s->num_restarts = num_restarts;
    return UG4GB_OK;
}

int ug4gb_solver_set_min_orthogonality(ug4gb_solver *s, double min_ortho)
{
    if (!s || !(min_ortho >= 0.0) || s->kind != UG4GB_SOLVER_BICGSTAB) return UG4GB_ERR_INVALID;
    s->min_ortho = min_ortho;
    return UG4GB_OK;
}

int ug4gb_solver_init(ug4gb_solver *s, const ug4gb_matrix *A)
{
    ug4gb::NvtxRange nvtx_("ug4gb:solver_init");
    if (!s || !A || A->A.nrows != A->A.ncols) return UG4GB_ERR_INVALID;
    return guarded(s->ctx, [&] {
        ug4gb_matrix *Am = const_cast<ug4gb_matrix *>(A);
        Am->ensure_op();
        // the same operator refreshed in place (same buffers, same layout) and
        // the same vectors: the captured iteration graph stays valid
        const uint64_t sig = op_signature(A->op);
        const bool same = (s->A == A && s->n == A->A.nrows && s->op_sig == sig);
        if (!same) drop_graph(s);
        s->A = A;
        s->op_sig = sig;
        s->n = A->A.nrows;
        size_t n = s->n > 0 ? s->n : 1;
        s->p.alloc(n);
        s->q.alloc(n);
        s->r.alloc(n);
        if (s->kind == UG4GB_SOLVER_BICGSTAB) {
            s->r0.alloc(n);
            s->v.alloc(n);
            s->s.alloc(n);
            s->t.alloc(n);
        }
    });
}

int ug4gb_solver_apply_return_defect(ug4gb_solver *s, ug4gb_vector *x, ug4gb_vector *b)
{
    ug4gb::NvtxRange nvtx_("ug4gb:solver_apply_return_defect");
    if (!s || !x || !b || x->n != s->n || b->n != s->n) return UG4GB_ERR_INVALID;
    return guarded(s->ctx, [&] { run(s, x->d, b->d); });
}

int ug4gb_solver_apply(ug4gb_solver *s, ug4gb_vector *x, const ug4gb_vector *b)
{
    ug4gb::NvtxRange nvtx_("ug4gb:solver_apply");
    if (!s || !x || !b || x->n != s->n || b->n != s->n) return UG4GB_ERR_INVALID;
    return guarded(s->ctx, [&] {
        UG_CUDA(cudaMemcpyAsync(s->r.p, b->d, sizeof(double) * (size_t)s->n, cudaMemcpyDeviceToDevice,
                                s->ctx->c.stream));
        run(s, x->d, s->r.p);
    });
}

int ug4gb_solver_solve_host(ug4gb_solver *s, const double *b_host, double *x_host)
{
    ug4gb::NvtxRange nvtx_("ug4gb:solver_solve_host");
    if (!s || !b_host || !x_host) return UG4GB_ERR_INVALID;
    return guarded(s->ctx, [&] {
        Ctx &c = s->ctx->c;
        if (!s->zcopy.p || (int)s->zcopy.n != s->n) s->zcopy.alloc(s->n > 0 ? s->n : 1);
        UG_CUDA(cudaMemcpyAsync(s->r.p, b_host, sizeof(double) * (size_t)s->n, cudaMemcpyHostToDevice, c.stream));
        UG_CUDA(cudaMemsetAsync(s->zcopy.p, 0, sizeof(double) * (size_t)s->n, c.stream));
        int rc_inner = UG4GB_OK;
        try {
            run(s, s->zcopy.p, s->r.p);
        } catch (const Error &e) {
            rc_inner = e.code;
            c.err = e.msg;
        }
        UG_CUDA(cudaMemcpyAsync(x_host, s->zcopy.p, sizeof(double) * (size_t)s->n, cudaMemcpyDeviceToHost, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        if (rc_inner != UG4GB_OK) throw Error{rc_inner, c.err};
    });
}

int ug4gb_solver_get_stats(const ug4gb_solver *s, int *steps, double *d0, double *d1, int *converged)
{
    if (!s) return UG4GB_ERR_INVALID;
    const KScal &k = s->host_ks;
    if (steps) *steps = k.step;
    if (d0) *d0 = k.d0;
    if (d1) *d1 = k.dcur;
    if (converged) *converged = (k.dcur < k.min_def) || (k.dcur / k.d0 < k.rel_red);
    return UG4GB_OK;
}

int ug4gb_solver_get_history(const ug4gb_solver *s, double *hist, int cap)
{
    if (!s || !hist) return UG4GB_ERR_INVALID;
    int n = (int)s->host_hist.size() < cap ? (int)s->host_hist.size() : cap;
    std::memcpy(hist, s->host_hist.data(), sizeof(double) * (size_t)n);
    return n;
}

void ug4gb_solver_destroy(ug4gb_solver *s)
{
    if (!s) return;
    ug4gb_ctx *ctx = s->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    drop_graph(s);
    free_pinned(s);
    delete s;
    ug4gb_ctx_release(ctx);
}

}  // extern "C"
