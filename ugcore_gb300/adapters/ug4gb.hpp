// ug4gb.hpp -- header-only C++ RAII layer over the C ABI (include/ug4gb.h).
//
// Every call checks its status and throws ug4gb::Error with the library's
// message; ugcore-side glue (ugcore_gpu_algebra.h) turns that into UG_THROW.
#pragma once

#include <cstdint>
#include <algorithm>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ug4gb.h"

namespace ug4gb {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc, const ug4gb_ctx *ctx, const char *what)
{
    if (rc != UG4GB_OK)
        throw Error(rc, std::string(what) + ": " + (ctx ? ug4gb_last_error(ctx) : "invalid handle"));
}

template <class H, void (*Destroy)(H *)>
class Handle {
public:
    Handle() = default;
    explicit Handle(H *h) : h_(h) {}
    Handle(const Handle &) = delete;
    Handle &operator=(const Handle &) = delete;
    Handle(Handle &&o) noexcept : h_(o.h_) { o.h_ = nullptr; }
    Handle &operator=(Handle &&o) noexcept
    {
        if (this != &o) { reset(); h_ = o.h_; o.h_ = nullptr; }
        return *this;
    }
    ~Handle() { reset(); }
    void reset()
    {
        if (h_) Destroy(h_);
        h_ = nullptr;
    }
    H *get() const { return h_; }

private:
    H *h_ = nullptr;
};

class Context {
public:
    explicit Context(int device = 0)
    {
        ug4gb_ctx *c = nullptr;
        int rc = ug4gb_create(device, &c);
        if (rc != UG4GB_OK) throw Error(rc, "ug4gb_create failed (no usable CUDA device?)");
        h_ = decltype(h_)(c);
    }
    ug4gb_ctx *get() const { return h_.get(); }
    void synchronize() const { check(ug4gb_synchronize(get()), get(), "synchronize"); }

private:
    Handle<ug4gb_ctx, ug4gb_destroy> h_;
};

class Grid {
public:
    Grid(const Context &c, int elem_type, int mx, int my, int mz, int nref) : ctx_(c.get())
    {
        ug4gb_grid *g = nullptr;
        check(ug4gb_grid_create_structured(ctx_, elem_type, mx, my, mz, nref, &g), ctx_, "grid");
        h_ = decltype(h_)(g);
    }
    ug4gb_grid *get() const { return h_.get(); }
    int num_levels() const { return ug4gb_grid_num_levels(get()); }
    int num_vertices(int level) const
    {
        int nv = 0;
        check(ug4gb_grid_level_info(get(), level, &nv, nullptr, nullptr, nullptr), ctx_, "grid info");
        return nv;
    }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_grid, ug4gb_grid_destroy> h_;
};

class Vector {
public:
    Vector(ug4gb_ctx *ctx, int n) : ctx_(ctx)
    {
        ug4gb_vector *v = nullptr;
        check(ug4gb_vector_create(ctx, n, &v), ctx, "vector");
        h_ = decltype(h_)(v);
    }
    ug4gb_vector *get() const { return h_.get(); }
    ug4gb_ctx *ctx() const { return ctx_; }
    int size() const { return ug4gb_vector_size(get()); }
    void set(double v) { check(ug4gb_vector_set(get(), v), ctx_, "vector set"); }
    void copy_from(const double *src) { check(ug4gb_vector_copy_from(get(), src), ctx_, "vector copy_from"); }
    void copy_to(double *dst) const { check(ug4gb_vector_copy_to(get(), dst), ctx_, "vector copy_to"); }
    double norm() const
    {
        double r = 0.0;
        check(ug4gb_vector_norm(get(), &r), ctx_, "vector norm");
        return r;
    }
    double dot(const Vector &o) const
    {
        double r = 0.0;
        check(ug4gb_vector_dot(get(), o.get(), &r), ctx_, "vector dot");
        return r;
    }
    // this = a*x + b*y
    void scale_add(double a, const Vector &x, double b, const Vector &y)
    {
        check(ug4gb_vector_scale_add(get(), a, x.get(), b, y.get()), ctx_, "vector scale_add");
    }
    double maxnorm() const
    {
        double r = 0.0;
        check(ug4gb_vector_maxnorm(get(), &r), ctx_, "vector maxnorm");
        return r;
    }
    double get_value(int i) const
    {
        double v = 0.0;
        check(ug4gb_vector_get_values(get(), 1, &i, &v), ctx_, "vector get");
        return v;
    }
    void set_value(int i, double v) { check(ug4gb_vector_set_values(get(), 1, &i, &v), ctx_, "vector set value"); }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_vector, ug4gb_vector_destroy> h_;
};

class Matrix {
public:
    explicit Matrix(ug4gb_ctx *ctx) : ctx_(ctx)
    {
        ug4gb_matrix *m = nullptr;
        check(ug4gb_matrix_create(ctx, &m), ctx, "matrix");
        h_ = decltype(h_)(m);
    }
    ug4gb_matrix *get() const { return h_.get(); }
    ug4gb_ctx *ctx() const { return ctx_; }
    void info(int &rows, int &cols, int64_t &nnz) const
    {
        check(ug4gb_matrix_info(get(), &rows, &cols, &nnz), ctx_, "matrix info");
    }
    void set_csr(int rows, int cols, const std::vector<int> &rp, const std::vector<int> &ci,
                 const std::vector<double> &va)
    {
        check(ug4gb_matrix_set_csr(get(), rows, cols, (int64_t)ci.size(), rp.data(), ci.data(), va.data()), ctx_,
              "matrix set_csr");
    }
    void axpy(Vector &dest, double a, const Vector *v1, double b, const Vector &w1) const
    {
        check(ug4gb_matrix_axpy(get(), dest.get(), a, v1 ? v1->get() : nullptr, b, w1.get()), ctx_, "matrix axpy");
    }
    void axpy_transposed(Vector &dest, double a, const Vector *v1, double b, const Vector &w1) const
    {
        check(ug4gb_matrix_axpy_transposed(get(), dest.get(), a, v1 ? v1->get() : nullptr, b, w1.get()), ctx_,
              "matrix axpy_transposed");
    }
    void set_as_transpose_of(const Matrix &B, bool keep_zeros = true)
    {
        check(ug4gb_matrix_set_as_transpose_of(get(), B.get(), keep_zeros ? 1 : 0), ctx_, "transpose");
    }
    void resize_and_clear(int rows, int cols)
    {
        check(ug4gb_matrix_resize_and_clear(get(), rows, cols), ctx_, "resize_and_clear");
    }
    void clear_retain_structure() { check(ug4gb_matrix_clear_retain_structure(get()), ctx_, "clear values"); }
    void set_as_copy_of(const Matrix &B, double scale = 1.0)
    {
        check(ug4gb_matrix_set_as_copy_of(get(), B.get(), scale), ctx_, "set_as_copy_of");
    }
    void scale(double a) { check(ug4gb_matrix_scale(get(), a), ctx_, "matrix scale"); }
    void apply_ignore_zero_rows(Vector &dest, double beta, const Vector &w) const
    {
        check(ug4gb_matrix_apply_ignore_zero_rows(get(), dest.get(), beta, w.get()), ctx_, "apply_ignore_zero_rows");
    }
    // row r copied to the host
    void row(int r, std::vector<int> &cols, std::vector<double> &vals) const
    {
        const int n = ug4gb_matrix_get_row(get(), r, nullptr, nullptr, 0);
        if (n < 0) check(n, ctx_, "matrix row");
        cols.resize(n);
        vals.resize(n);
        if (n > 0) check(std::min(0, ug4gb_matrix_get_row(get(), r, cols.data(), vals.data(), n)), ctx_, "matrix row");
    }
    void add_entries(const std::vector<int> &rows, const std::vector<int> &cols, const std::vector<double> &vals)
    {
        check(ug4gb_matrix_add_entries(get(), (int)rows.size(), rows.data(), cols.data(), vals.data()), ctx_,
              "add_entries");
    }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_matrix, ug4gb_matrix_destroy> h_;
};

class Disc {
public:
    Disc(const Context &c, const Grid &g) : ctx_(c.get())
    {
        ug4gb_disc *d = nullptr;
        check(ug4gb_disc_create(ctx_, g.get(), &d), ctx_, "disc");
        h_ = decltype(h_)(d);
    }
    ug4gb_disc *get() const { return h_.get(); }
    void set_diffusion(double K) { check(ug4gb_disc_set_diffusion_constant(get(), K), ctx_, "set_diffusion"); }
    void set_source_uniform(uint64_t seed) { check(ug4gb_disc_set_source_uniform(get(), seed), ctx_, "source"); }
    void set_source(const double *f) { check(ug4gb_disc_set_source_vertices(get(), f), ctx_, "source"); }
    void assemble_linear(int level, Matrix &A, Vector &b)
    {
        check(ug4gb_disc_assemble_linear(get(), level, A.get(), b.get()), ctx_, "assemble_linear");
    }
    void assemble_jacobian(int level, Matrix &A)
    {
        check(ug4gb_disc_assemble_jacobian(get(), level, A.get()), ctx_, "assemble_jacobian");
    }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_disc, ug4gb_disc_destroy> h_;
};

class GMG {
public:
    GMG(const Context &c, Disc &d) : ctx_(c.get())
    {
        ug4gb_gmg *m = nullptr;
        check(ug4gb_gmg_create(ctx_, d.get(), &m), ctx_, "gmg");
        h_ = decltype(h_)(m);
    }
    ug4gb_gmg *get() const { return h_.get(); }
    void set_smoother(int kind, double damp) { check(ug4gb_gmg_set_smoother(get(), kind, damp), ctx_, "smoother"); }
    void set_cycle_type(int c) { check(ug4gb_gmg_set_cycle_type(get(), c), ctx_, "cycle"); }
    void set_num_presmooth(int n) { check(ug4gb_gmg_set_num_presmooth(get(), n), ctx_, "presmooth"); }
    void set_num_postsmooth(int n) { check(ug4gb_gmg_set_num_postsmooth(get(), n), ctx_, "postsmooth"); }
    void set_base_level(int l) { check(ug4gb_gmg_set_base_level(get(), l), ctx_, "base level"); }
    void set_precision(int p) { check(ug4gb_gmg_set_precision(get(), p), ctx_, "precision"); }
    void init(const Matrix &A) { check(ug4gb_gmg_init(get(), A.get()), ctx_, "gmg init"); }
    void apply(Vector &c, const Vector &d) { check(ug4gb_gmg_apply(get(), c.get(), d.get()), ctx_, "gmg apply"); }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_gmg, ug4gb_gmg_destroy> h_;
};

class Solver {
public:
    Solver(const Context &c, int kind) : ctx_(c.get())
    {
        ug4gb_solver *s = nullptr;
        check(ug4gb_solver_create(ctx_, kind, &s), ctx_, "solver");
        h_ = decltype(h_)(s);
    }
    ug4gb_solver *get() const { return h_.get(); }
    void set_preconditioner(GMG *m) { check(ug4gb_solver_set_preconditioner(get(), m ? m->get() : nullptr), ctx_, "pre"); }
    void set_convergence_check(int maxit, double min_def, double red)
    {
        check(ug4gb_solver_set_convergence_check(get(), maxit, min_def, red), ctx_, "convcheck");
    }
    void init(const Matrix &A) { check(ug4gb_solver_init(get(), A.get()), ctx_, "solver init"); }
    // returns false if not converged (like ILinearOperatorInverse::apply)
    bool apply_return_defect(Vector &x, Vector &b)
    {
        int rc = ug4gb_solver_apply_return_defect(get(), x.get(), b.get());
        if (rc == UG4GB_ERR_NOT_CONVERGED || rc == UG4GB_ERR_BREAKDOWN) return false;
        check(rc, ctx_, "solver apply");
        return true;
    }
    bool apply(Vector &x, const Vector &b)
    {
        int rc = ug4gb_solver_apply(get(), x.get(), b.get());
        if (rc == UG4GB_ERR_NOT_CONVERGED || rc == UG4GB_ERR_BREAKDOWN) return false;
        check(rc, ctx_, "solver apply");
        return true;
    }
    int steps() const
    {
        int s = 0;
        ug4gb_solver_get_stats(get(), &s, nullptr, nullptr, nullptr);
        return s;
    }
    double defect() const
    {
        double d = 0.0;
        ug4gb_solver_get_stats(get(), nullptr, nullptr, &d, nullptr);
        return d;
    }

private:
    ug4gb_ctx *ctx_;
    Handle<ug4gb_solver, ug4gb_solver_destroy> h_;
};

}  // namespace ug4gb
