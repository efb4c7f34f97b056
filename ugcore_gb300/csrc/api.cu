// api.cu -- C ABI: context, grid hierarchy, vectors, matrices.
#include <atomic>
#include <cstring>

#include "gmg.cuh"

using namespace ug4gb;

namespace ug4gb {

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

void copy_in(Ctx &c, void *dst_dev, const void *src, size_t bytes)
{
    if (!bytes) return;
    UG_CUDA(cudaMemcpyAsync(dst_dev, src, bytes, cudaMemcpyDefault, c.stream));
}

void copy_out(Ctx &c, void *dst, const void *src_dev, size_t bytes)
{
    if (!bytes) return;
    UG_CUDA(cudaMemcpyAsync(dst, src_dev, bytes, cudaMemcpyDefault, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

void gen_level(Ctx &c, Level &L, int elem_type, int cx, int cy, int cz, const Level *coarse);

cudaEvent_t prof_event(Ctx &c)
{
    cudaEvent_t e;
    if (!c.ev_pool.empty()) {
        e = c.ev_pool.back();
        c.ev_pool.pop_back();
    } else {
        UG_CUDA(cudaEventCreate(&e));
    }
    return e;
}

}  // namespace ug4gb

// Runs f, translating internal errors into status codes (no exception
// crosses the C boundary).
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

extern "C" {

int ug4gb_create(int device, ug4gb_ctx **out)
{
    if (!out) return UG4GB_ERR_INVALID;
    *out = nullptr;
    ug4gb_ctx *ctx = new ug4gb_ctx;
    int rc = guarded(ctx, [&] {
        int ndev = 0;
        UG_CUDA(cudaGetDeviceCount(&ndev));
        UG_REQUIRE(device >= 0 && device < ndev, UG4GB_ERR_INVALID, "ug4gb_create: no such CUDA device");
        UG_CUDA(cudaSetDevice(device));
        Ctx &c = ctx->c;
        c.device = device;
        UG_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
        UG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        c.red_partials.alloc((size_t)kRedMaxBlocks * kRedMaxValues);
        c.red_counter.alloc(64);
        c.red_result.alloc(8);
        c.dev_err.alloc(1);
        UG_CUDA(cudaMemset(c.red_counter.p, 0, c.red_counter.bytes()));
        UG_CUDA(cudaMemset(c.dev_err.p, 0, sizeof(int)));
        UG_CUDA(cudaMallocHost((void **)&c.host_pinned, 256));
    });
    if (rc != UG4GB_OK) {
        delete ctx;
        return rc;
    }
    *out = ctx;
    return UG4GB_OK;
}

void ug4gb_ctx_retain(ug4gb_ctx *ctx)
{
    if (ctx) ctx->refs++;
}

static void ctx_free(ug4gb_ctx *ctx);

void ug4gb_ctx_release(ug4gb_ctx *ctx)
{
    if (ctx && --ctx->refs == 0) ctx_free(ctx);
}

void ug4gb_destroy(ug4gb_ctx *ctx)
{
    if (!ctx || ctx->closed) return;
    ctx->closed = true;
    ug4gb_ctx_release(ctx);
}

static void ctx_free(ug4gb_ctx *ctx)
{
    cudaSetDevice(ctx->c.device);
    if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
    if (ctx->c.host_pinned) cudaFreeHost(ctx->c.host_pinned);
    for (auto &r : ctx->c.prof) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : ctx->c.ev_pool) cudaEventDestroy(e);
    ctx->c.red_partials.release();
    ctx->c.red_counter.release();
    ctx->c.red_result.release();
    ctx->c.dev_err.release();
    if (ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
    delete ctx;
}

const char *ug4gb_last_error(const ug4gb_ctx *ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int ug4gb_synchronize(ug4gb_ctx *ctx)
{
    if (!ctx) return UG4GB_ERR_INVALID;
    return guarded(ctx, [&] { UG_CUDA(cudaStreamSynchronize(ctx->c.stream)); });
}

void *ug4gb_stream(ug4gb_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int64_t ug4gb_kernel_launches(const ug4gb_ctx *ctx) { return ctx ? ctx->c.launches : -1; }

int ug4gb_set_operator_format(ug4gb_ctx *ctx, int format)
{
    if (!ctx || (format != UG4GB_FORMAT_AUTO && format != UG4GB_FORMAT_SELL)) return UG4GB_ERR_INVALID;
    ctx->c.allow_dia = (format == UG4GB_FORMAT_AUTO);
    return UG4GB_OK;
}

int ug4gb_set_tuning(ug4gb_ctx *ctx, int knob, int value)
{
    if (!ctx) return UG4GB_ERR_INVALID;
    switch (knob) {
    case UG4GB_TUNE_PDL:
        if (value != 0 && value != 1) return UG4GB_ERR_INVALID;
        ctx->c.pdl = value != 0;
        return UG4GB_OK;
    case UG4GB_TUNE_SWEEP_FUSION:
        if (value < 0 || value > 3) return UG4GB_ERR_INVALID;
        ctx->c.sweep_fusion = value;
        return UG4GB_OK;
    case UG4GB_TUNE_SWEEP_PLANES:
        if (value < 2 || value > 128) return UG4GB_ERR_INVALID;
        ctx->c.sweep_fusion_tz = value;
        return UG4GB_OK;
    case UG4GB_TUNE_SWEEP_WAIT_TEST:
        if (value < 0 || value > 4096 || value % 16) return UG4GB_ERR_INVALID;
        ctx->c.sweep_wait_test = value;
        return UG4GB_OK;
    case UG4GB_TUNE_COARSE_LEVELS:
        if (value < -1 || value > 7) return UG4GB_ERR_INVALID;
        ctx->c.coarse_levels = value;
        return UG4GB_OK;
    case UG4GB_TUNE_ROW_ASSEMBLY:
        if (value < 0 || value > 2) return UG4GB_ERR_INVALID;
        ctx->c.row_assembly = value;
        return UG4GB_OK;
    default: ctx->c.err = "ug4gb_set_tuning: unknown knob"; return UG4GB_ERR_INVALID;
    }
}

int ug4gb_profile_begin(ug4gb_ctx *ctx)
{
    if (!ctx) return UG4GB_ERR_INVALID;
    return guarded(ctx, [&] {
        UG_CUDA(cudaStreamSynchronize(ctx->c.stream));
        for (auto &r : ctx->c.prof) {
            ctx->c.ev_pool.push_back(r.a);
            ctx->c.ev_pool.push_back(r.b);
        }
        ctx->c.prof.clear();
        ctx->c.profiling = true;
    });
}

int ug4gb_profile_end(ug4gb_ctx *ctx, char *buf, int cap)
{
    if (!ctx || !buf || cap <= 0) return UG4GB_ERR_INVALID;
    return guarded(ctx, [&] {
        Ctx &c = ctx->c;
        UG_CUDA(cudaStreamSynchronize(c.stream));
        c.profiling = false;
        std::vector<std::pair<std::string, std::pair<int, double>>> acc;
        for (auto &r : c.prof) {
            float ms = 0.f;
            UG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
            size_t i = 0;
            for (; i < acc.size(); ++i)
                if (acc[i].first == r.name) break;
            if (i == acc.size()) acc.push_back({r.name, {0, 0.0}});
            acc[i].second.first += 1;
            acc[i].second.second += ms;
            c.ev_pool.push_back(r.a);
            c.ev_pool.push_back(r.b);
        }
        c.prof.clear();
        std::string out;
        for (auto &a : acc) {
            char line[512];
            snprintf(line, sizeof(line), "%s\t%d\t%.6f\n", a.first.c_str(), a.second.first, a.second.second);
            out += line;
        }
        int n = (int)out.size() < cap - 1 ? (int)out.size() : cap - 1;
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    });
}

// ------------------------------------------------------------------ grid --
uint64_t ug4gb_next_grid_uid()
{
    static std::atomic<uint64_t> next{1};
    return next.fetch_add(1, std::memory_order_relaxed);
}

int ug4gb_grid_create_structured(ug4gb_ctx *ctx, int elem_type, int mx, int my, int mz, int nref, ug4gb_grid **out)
{
    if (!ctx || !out) return UG4GB_ERR_INVALID;
    *out = nullptr;
    ug4gb_grid *g = new ug4gb_grid;
    int rc = guarded(ctx, [&] {
        UG_REQUIRE(elem_type >= UG4GB_QUAD && elem_type <= UG4GB_TET, UG4GB_ERR_INVALID, "grid: bad element type");
        UG_REQUIRE(mx >= 1 && my >= 1 && (elem_type == UG4GB_QUAD || mz >= 1), UG4GB_ERR_INVALID,
                   "grid: coarse cell counts must be >= 1");
        UG_REQUIRE(nref >= 0 && nref <= 12, UG4GB_ERR_INVALID, "grid: refinement count out of range");
        const double fr = (double)(1 << nref);
        double nv = ((double)mx * fr + 1) * ((double)my * fr + 1) * (elem_type == UG4GB_QUAD ? 1.0 : (double)mz * fr + 1);
        UG_REQUIRE(nv < 2.0e9, UG4GB_ERR_INVALID, "grid: too many vertices for 32-bit indices");
        // element corner lists are indexed with 32 bits: ne * corners < 2^31
        const double cells = (double)mx * fr * ((double)my * fr) * (elem_type == UG4GB_QUAD ? 1.0 : (double)mz * fr);
        const double corners = cells * (elem_type == UG4GB_TET ? 6.0 * 4.0 : (elem_type == UG4GB_HEX ? 8.0 : 4.0));
        UG_REQUIRE(corners < 2147483648.0, UG4GB_ERR_INVALID, "grid: too many element corners for 32-bit indices");
        g->ctx = ctx;
        g->elem_type = elem_type;
        g->lev.resize(nref + 1);
        for (int l = 0; l <= nref; ++l) {
            int f = 1 << l;
            gen_level(ctx->c, g->lev[l], elem_type, mx * f, my * f, mz * f, l > 0 ? &g->lev[l - 1] : nullptr);
        }
        UG_CUDA(cudaStreamSynchronize(ctx->c.stream));
    });
    if (rc != UG4GB_OK) {
        delete g;
        return rc;
    }
    ug4gb_ctx_retain(ctx);
    *out = g;
    return UG4GB_OK;
}

int ug4gb_grid_num_levels(const ug4gb_grid *g) { return g ? (int)g->lev.size() : UG4GB_ERR_INVALID; }

int ug4gb_grid_level_info(const ug4gb_grid *g, int level, int *nv, int *ne, int *k, int *dim)
{
    if (!g || level < 0 || level >= (int)g->lev.size()) return UG4GB_ERR_INVALID;
    const Level &L = g->lev[level];
    if (nv) *nv = L.nv;
    if (ne) *ne = L.ne;
    if (k) *k = L.k;
    if (dim) *dim = L.dim;
    return UG4GB_OK;
}

int ug4gb_grid_level_export(const ug4gb_grid *g, int level, double *coords, int *elems, unsigned char *bnd)
{
    if (!g || level < 0 || level >= (int)g->lev.size()) return UG4GB_ERR_INVALID;
    return guarded(g->ctx, [&] {
        const Level &L = g->lev[level];
        Ctx &c = g->ctx->c;
        if (coords) copy_out(c, coords, L.coords.p, L.coords.bytes());
        if (elems) copy_out(c, elems, L.elems.p, L.elems.bytes());
        if (bnd) copy_out(c, bnd, L.bnd.p, L.bnd.bytes());
    });
}

void ug4gb_grid_destroy(ug4gb_grid *g)
{
    if (!g) return;
    ug4gb_ctx *ctx = g->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete g;
    ug4gb_ctx_release(ctx);
}

// --------------------------------------------------------------- vectors --
int ug4gb_vector_create(ug4gb_ctx *ctx, int n, ug4gb_vector **out)
{
    if (!ctx || !out || n < 0) return UG4GB_ERR_INVALID;
    *out = nullptr;
    ug4gb_vector *v = new ug4gb_vector;
    int rc = guarded(ctx, [&] {
        v->ctx = ctx;
        v->n = n;
        v->own.alloc(n > 0 ? n : 1);
        v->d = v->own.p;
        UG_CUDA(cudaMemsetAsync(v->d, 0, sizeof(double) * (size_t)(n > 0 ? n : 1), ctx->c.stream));
    });
    if (rc != UG4GB_OK) {
        delete v;
        return rc;
    }
    ug4gb_ctx_retain(ctx);
    *out = v;
    return UG4GB_OK;
}

int ug4gb_vector_wrap(ug4gb_ctx *ctx, double *dptr, int n, ug4gb_vector **out)
{
    if (!ctx || !out || n < 0 || (n > 0 && !dptr)) return UG4GB_ERR_INVALID;
    if (n > 0 && !is_device_ptr(dptr)) {
        ctx->c.err = "ug4gb_vector_wrap: pointer is not device memory";
        return UG4GB_ERR_INVALID;
    }
    ug4gb_vector *v = new ug4gb_vector;
    v->ctx = ctx;
    v->n = n;
    v->d = dptr;
    ug4gb_ctx_retain(ctx);
    *out = v;
    return UG4GB_OK;
}

int ug4gb_vector_size(const ug4gb_vector *v) { return v ? v->n : UG4GB_ERR_INVALID; }
double *ug4gb_vector_data(ug4gb_vector *v) { return v ? v->d : nullptr; }

int ug4gb_vector_set(ug4gb_vector *v, double value)
{
    if (!v) return UG4GB_ERR_INVALID;
    return guarded(v->ctx, [&] { fill_double(v->ctx->c, v->d, v->n, value); });
}

int ug4gb_vector_copy_from(ug4gb_vector *v, const double *src)
{
    if (!v || (!src && v->n)) return UG4GB_ERR_INVALID;
    return guarded(v->ctx, [&] { copy_in(v->ctx->c, v->d, src, sizeof(double) * (size_t)v->n); });
}

int ug4gb_vector_copy_to(const ug4gb_vector *v, double *dst)
{
    if (!v || (!dst && v->n)) return UG4GB_ERR_INVALID;
    return guarded(v->ctx, [&] { copy_out(v->ctx->c, dst, v->d, sizeof(double) * (size_t)v->n); });
}

static int dot_impl(const ug4gb_vector *a, const ug4gb_vector *b, double *out)
{
    Ctx &c = a->ctx->c;
    return guarded(a->ctx, [&] {
        DevBuf<KScal> ks;
        ks.alloc(1);
        RedArgs red{c.red_partials.p, c.red_counter.p + 8, ks.p};
        vec_dot(c, a->n, a->d, b->d, red);
        KScal h;
        copy_out(c, &h, ks.p, sizeof(KScal));
        *out = h.dot_out[0];
    });
}

int ug4gb_vector_norm(const ug4gb_vector *v, double *out)
{
    if (!v || !out) return UG4GB_ERR_INVALID;
    double s = 0.0;
    int rc = dot_impl(v, v, &s);
    *out = sqrt(s);
    return rc;
}

int ug4gb_vector_dot(const ug4gb_vector *a, const ug4gb_vector *b, double *out)
{
    if (!a || !b || !out || a->n != b->n) return UG4GB_ERR_INVALID;
    return dot_impl(a, b, out);
}

int ug4gb_vector_scale_add(ug4gb_vector *dest, double alpha, const ug4gb_vector *a, double beta, const ug4gb_vector *b)
{
    if (!dest || !a || !b || a->n != dest->n || b->n != dest->n) return UG4GB_ERR_INVALID;
    return guarded(dest->ctx, [&] { vec_scale_add(dest->ctx->c, dest->n, dest->d, alpha, a->d, beta, b->d); });
}

void ug4gb_vector_destroy(ug4gb_vector *v)
{
    if (!v) return;
    ug4gb_ctx *ctx = v->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete v;
    ug4gb_ctx_release(ctx);
}

// -------------------------------------------------------------- matrices --
int ug4gb_matrix_create(ug4gb_ctx *ctx, ug4gb_matrix **out)
{
    if (!ctx || !out) return UG4GB_ERR_INVALID;
    ug4gb_matrix *m = new ug4gb_matrix;
    m->ctx = ctx;
    ug4gb_ctx_retain(ctx);
    *out = m;
    return UG4GB_OK;
}

int ug4gb_matrix_set_csr(ug4gb_matrix *m, int nrows, int ncols, int64_t nnz, const int *rowptr, const int *col,
                         const double *val)
{
    if (!m || nrows < 0 || ncols < 0 || nnz < 0 || !rowptr || (nnz && (!col || !val))) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        m->A.nrows = nrows;
        m->A.ncols = ncols;
        m->A.nnz = nnz;
        m->A.rowptr.alloc(nrows + 1);
        m->A.col.alloc(nnz > 0 ? nnz : 1);
        m->A.val.alloc(nnz > 0 ? nnz : 1);
        copy_in(c, m->A.rowptr.p, rowptr, sizeof(int) * (size_t)(nrows + 1));
        copy_in(c, m->A.col.p, col, sizeof(int) * (size_t)nnz);
        copy_in(c, m->A.val.p, val, sizeof(double) * (size_t)nnz);
        UG_CUDA(cudaStreamSynchronize(c.stream));
        m->op_valid = false;
        m->pattern_grid = 0;
        m->derived_key = 0;
        m->pattern_level = -1;
    });
}

int ug4gb_matrix_info(const ug4gb_matrix *m, int *nrows, int *ncols, int64_t *nnz)
{
    if (!m) return UG4GB_ERR_INVALID;
    if (nrows) *nrows = m->A.nrows;
    if (ncols) *ncols = m->A.ncols;
    if (nnz) *nnz = m->A.nnz;
    return UG4GB_OK;
}

int ug4gb_matrix_export_csr(const ug4gb_matrix *m, int *rowptr, int *col, double *val)
{
    if (!m) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        if (rowptr) copy_out(c, rowptr, m->A.rowptr.p, sizeof(int) * (size_t)(m->A.nrows + 1));
        if (col) copy_out(c, col, m->A.col.p, sizeof(int) * (size_t)m->A.nnz);
        if (val) copy_out(c, val, m->A.val.p, sizeof(double) * (size_t)m->A.nnz);
    });
}

int ug4gb_matrix_axpy(const ug4gb_matrix *mc, ug4gb_vector *dest, double alpha1, const ug4gb_vector *v1, double beta1,
                      const ug4gb_vector *w1)
{
    ug4gb_matrix *m = const_cast<ug4gb_matrix *>(mc);
    if (!m || !dest || !w1 || dest->n != m->A.nrows || w1->n != m->A.ncols) return UG4GB_ERR_INVALID;
    if (alpha1 != 0.0 && (!v1 || v1->n != m->A.nrows)) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        m->ensure_op();
        op_axpy(m->ctx->c, m->op, dest->d, alpha1, alpha1 != 0.0 ? v1->d : dest->d, beta1, w1->d);
    });
}

int ug4gb_matrix_axpy_transposed(const ug4gb_matrix *m, ug4gb_vector *dest, double alpha1, const ug4gb_vector *v1,
                                 double beta1, const ug4gb_vector *w1)
{
    if (!m || !dest || !w1 || dest->n != m->A.ncols || w1->n != m->A.nrows) return UG4GB_ERR_INVALID;
    if (alpha1 != 0.0 && (!v1 || v1->n != m->A.ncols)) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        if (alpha1 == 0.0) fill_double(c, dest->d, dest->n, 0.0);
        else if (!(v1 == dest && alpha1 == 1.0)) vec_scale_add(c, dest->n, dest->d, alpha1, v1->d, 0.0, v1->d);
        csr_axpy_transposed(c, m->A, dest->d, beta1, w1->d);
    });
}

int ug4gb_matrix_set_as_transpose_of(ug4gb_matrix *T, const ug4gb_matrix *B, int keep_zeros)
{
    if (!T || !B || T == B) return UG4GB_ERR_INVALID;
    return guarded(T->ctx, [&] {
        csr_transpose(T->ctx->c, B->A, T->A, keep_zeros != 0);
        UG_CUDA(cudaStreamSynchronize(T->ctx->c.stream));
        T->op_valid = false;
        T->pattern_grid = 0;
        T->derived_key = 0;
        T->pattern_level = -1;
    });
}

void ug4gb_matrix_destroy(ug4gb_matrix *m)
{
    if (!m) return;
    ug4gb_ctx *ctx = m->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete m;
    ug4gb_ctx_release(ctx);
}

}  // extern "C"
