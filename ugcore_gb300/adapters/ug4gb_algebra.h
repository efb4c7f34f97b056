// ug4gb_algebra.h -- the ugcore-side GPU algebra type over libug4gb.
//
// A ugcore build with UG_GPU/UG4GB defined includes this header where the
// algebra types live (lib_algebra/cpu_algebra_types.h:103-119 keeps the slot
// for a GPU algebra) and adds GPUAlgebra to CompileAlgebraList
// (bridge/util_algebra_dependent.h:60-62); every RegisterAlgebraDependent
// then registers the "GPU1"-suffixed classes.  The types here follow the
// subsets of ug::Vector (lib_algebra/cpu_algebra/vector.h:54-230) and
// ug::SparseMatrix (lib_algebra/cpu_algebra/sparsematrix.h:98-330) that the
// Krylov solvers and linear operators use, forwarding to the C ABI through
// the RAII layer ug4gb.hpp.  Library errors become ugcore errors (UG_THROW).
//
// Needs ugcore's lib_algebra/algebra_type.h and common/error.h on the include
// path (the header is checked against them where the ugcore tree is present).
#pragma once

#include <memory>
#include <vector>

#include "common/error.h"
#include "common/util/smart_pointer.h"
#include "lib_algebra/algebra_type.h"
#include "ug4gb.hpp"

namespace ug {

namespace ug4gb_glue {

// one engine context per process: ugcore's hot path is single-threaded per rank
inline ug4gb::Context &context()
{
    static ug4gb::Context ctx(0);
    return ctx;
}

template <class F>
inline void guarded(F &&f, const char *what)
{
    try {
        f();
    } catch (const ug4gb::Error &e) {
        UG_THROW(what << ": " << e.what());
    }
}

}  // namespace ug4gb_glue

/// vector_type of GPUAlgebra: one device-resident FP64 vector
class UG4GBVector
{
public:
    typedef double value_type;
    typedef size_t size_type;

    UG4GBVector() = default;
    explicit UG4GBVector(size_t n) { resize(n); }
    UG4GBVector(const UG4GBVector &o) { *this = o; }
    UG4GBVector &operator=(const UG4GBVector &o)
    {
        if (this == &o) return *this;
        resize(o.size());
        if (size()) ug4gb_glue::guarded([&] { m_v->scale_add(1.0, *o.m_v, 0.0, *o.m_v); }, "UG4GBVector copy");
        return *this;
    }

    /// all entries = w (used as `v = 0.0` by the solvers)
    UG4GBVector &operator=(double w)
    {
        set(w);
        return *this;
    }

    void resize(size_t n)
    {
        if (n == size()) return;
        ug4gb_glue::guarded([&] { m_v.reset(new ug4gb::Vector(ug4gb_glue::context().get(), (int)n)); },
                            "UG4GBVector::resize");
    }
    size_t size() const { return m_v ? (size_t)m_v->size() : 0; }

    bool set(double w)
    {
        ug4gb_glue::guarded([&] { m_v->set(w); }, "UG4GBVector::set");
        return true;
    }
    double norm() const
    {
        double r = 0;
        ug4gb_glue::guarded([&] { r = m_v->norm(); }, "UG4GBVector::norm");
        return r;
    }
    double dotprod(const UG4GBVector &o) const
    {
        double r = 0;
        ug4gb_glue::guarded([&] { r = m_v->dot(*o.m_v); }, "UG4GBVector::dotprod");
        return r;
    }
    /// max |v_i| (Vector::maxnorm)
    double maxnorm() const
    {
        double r = 0;
        ug4gb_glue::guarded([&] { r = m_v->maxnorm(); }, "UG4GBVector::maxnorm");
        return r;
    }
    /// one entry read from the device (set-up and output code, not solver loops)
    double operator[](size_t i) const
    {
        double r = 0;
        ug4gb_glue::guarded([&] { r = m_v->get_value((int)i); }, "UG4GBVector::operator[]");
        return r;
    }
    /// one entry written on the device
    void set_value(size_t i, double v)
    {
        ug4gb_glue::guarded([&] { m_v->set_value((int)i, v); }, "UG4GBVector::set_value");
    }
    void copy_from_host(const double *src)
    {
        ug4gb_glue::guarded([&] { m_v->copy_from(src); }, "UG4GBVector::copy_from_host");
    }
    void copy_to_host(double *dst) const
    {
        ug4gb_glue::guarded([&] { m_v->copy_to(dst); }, "UG4GBVector::copy_to_host");
    }

    SmartPtr<UG4GBVector> clone() const { return SmartPtr<UG4GBVector>(new UG4GBVector(*this)); }
    SmartPtr<UG4GBVector> clone_without_values() const { return SmartPtr<UG4GBVector>(new UG4GBVector(size())); }

    UG4GBVector &operator+=(const UG4GBVector &o) { return axpby(1.0, o); }
    UG4GBVector &operator-=(const UG4GBVector &o) { return axpby(-1.0, o); }
    UG4GBVector &operator*=(double a)
    {
        ug4gb_glue::guarded([&] { m_v->scale_add(a, *m_v, 0.0, *m_v); }, "UG4GBVector *=");
        return *this;
    }

    ug4gb::Vector &impl() { return *m_v; }
    const ug4gb::Vector &impl() const { return *m_v; }

private:
    // this = 1 * this + b * o
    UG4GBVector &axpby(double b, const UG4GBVector &o)
    {
        ug4gb_glue::guarded([&] { m_v->scale_add(1.0, *m_v, b, *o.m_v); }, "UG4GBVector update");
        return *this;
    }
    std::shared_ptr<ug4gb::Vector> m_v;
};

/// matrix_type of GPUAlgebra: a device CRS (exported in ugcore's defragmented form)
class UG4GBSparseMatrix
{
public:
    typedef double value_type;

    UG4GBSparseMatrix()
    {
        ug4gb_glue::guarded([&] { m_A.reset(new ug4gb::Matrix(ug4gb_glue::context().get())); }, "UG4GBSparseMatrix");
    }

    size_t num_rows() const { return (size_t)info().r; }
    size_t num_cols() const { return (size_t)info().c; }
    size_t total_num_connections() const { return (size_t)info().nnz; }

    /// SparseMatrix::resize_and_clear (sparsematrix_impl.h:91): empty rows
    void resize_and_clear(size_t rows, size_t cols)
    {
        ug4gb_glue::guarded([&] { m_A->resize_and_clear((int)rows, (int)cols); }, "resize_and_clear");
    }
    /// SparseMatrix::clear_retain_structure (:142): values 0, pattern kept
    void clear_retain_structure()
    {
        ug4gb_glue::guarded([&] { m_A->clear_retain_structure(); }, "clear_retain_structure");
    }
    /// SparseMatrix::set_as_copy_of (:472): this = scale * B
    void set_as_copy_of(const UG4GBSparseMatrix &B, double scale = 1.0)
    {
        ug4gb_glue::guarded([&] { m_A->set_as_copy_of(*B.m_A, scale); }, "set_as_copy_of");
    }
    /// SparseMatrix::scale (:487)
    bool scale(double d)
    {
        ug4gb_glue::guarded([&] { m_A->scale(d); }, "scale");
        return true;
    }
    /// SparseMatrix::apply_ignore_zero_rows (:270-288): dest = beta A w on rows with stored entries
    void apply_ignore_zero_rows(UG4GBVector &dest, const double &beta1, const UG4GBVector &w1) const
    {
        ug4gb_glue::guarded([&] { m_A->apply_ignore_zero_rows(dest.impl(), beta1, w1.impl()); },
                            "apply_ignore_zero_rows");
    }
    /// A(r, c) read from the device (0 if not stored; set-up code, not solver loops)
    double operator()(size_t r, size_t c) const
    {
        std::vector<int> ci;
        std::vector<double> va;
        ug4gb_glue::guarded([&] { m_A->row((int)r, ci, va); }, "SparseMatrix::operator()");
        for (size_t a = 0; a < ci.size(); ++a)
            if (ci[a] == (int)c) return va[a];
        return 0.0;
    }
    /// element contributions added into the existing pattern (AddLocalMatrixToGlobal)
    void add_entries(const std::vector<int> &rows, const std::vector<int> &cols, const std::vector<double> &vals)
    {
        ug4gb_glue::guarded([&] { m_A->add_entries(rows, cols, vals); }, "add_entries");
    }

    /// CRS from host arrays (sorted columns per row, as SparseMatrix::defragment leaves them)
    void set_csr(int rows, int cols, const std::vector<int> &rowptr, const std::vector<int> &col,
                 const std::vector<double> &val)
    {
        ug4gb_glue::guarded([&] { m_A->set_csr(rows, cols, rowptr, col, val); }, "UG4GBSparseMatrix::set_csr");
    }

    /// dest = alpha1 v1 + beta1 A w1 (SparseMatrix::axpy, sparsematrix_impl.h:294)
    bool axpy(UG4GBVector &dest, const double &alpha1, const UG4GBVector &v1, const double &beta1,
              const UG4GBVector &w1) const
    {
        ug4gb_glue::guarded([&] { m_A->axpy(dest.impl(), alpha1, &v1.impl(), beta1, w1.impl()); },
                            "UG4GBSparseMatrix::axpy");
        return true;
    }
    /// dest = alpha1 v1 + beta1 A^T w1 (SparseMatrix::axpy_transposed, sparsematrix_impl.h:344)
    bool axpy_transposed(UG4GBVector &dest, const double &alpha1, const UG4GBVector &v1, const double &beta1,
                         const UG4GBVector &w1) const
    {
        ug4gb_glue::guarded([&] { m_A->axpy_transposed(dest.impl(), alpha1, &v1.impl(), beta1, w1.impl()); },
                            "UG4GBSparseMatrix::axpy_transposed");
        return true;
    }
    bool apply(UG4GBVector &f, const UG4GBVector &u) const { return axpy(f, 0.0, f, 1.0, u); }
    bool apply_transposed(UG4GBVector &f, const UG4GBVector &u) const { return axpy_transposed(f, 0.0, f, 1.0, u); }
    /// res -= A x
    bool matmul_minus(UG4GBVector &res, const UG4GBVector &x) const { return axpy(res, 1.0, res, -1.0, x); }
    /// this = B^T (SparseMatrix::set_as_transpose_of, sparsematrix_impl.h:149; zeros kept)
    void set_as_transpose_of(const UG4GBSparseMatrix &B)
    {
        ug4gb_glue::guarded([&] { m_A->set_as_transpose_of(*B.m_A, true); }, "set_as_transpose_of");
    }

    ug4gb::Matrix &impl() { return *m_A; }
    const ug4gb::Matrix &impl() const { return *m_A; }

private:
    struct Info {
        int r = 0, c = 0;
        int64_t nnz = 0;
    };
    Info info() const
    {
        Info i;
        ug4gb_glue::guarded([&] { m_A->info(i.r, i.c, i.nnz); }, "UG4GBSparseMatrix::info");
        return i;
    }
    std::shared_ptr<ug4gb::Matrix> m_A;
};

/// the algebra type (slot: lib_algebra/cpu_algebra_types.h:103-119; AlgebraType::GPU, algebra_type.h)
struct GPUAlgebra {
    typedef UG4GBSparseMatrix matrix_type;
    typedef UG4GBVector vector_type;
    static const int blockSize = 1;
    static AlgebraType get_type() { return AlgebraType(AlgebraType::GPU, 1); }
};

// the vector operations of lib_algebra/operations_vec.h:55-91 used by the Krylov solvers
inline void VecScaleAssign(UG4GBVector &d, double a, const UG4GBVector &x)
{
    ug4gb_glue::guarded([&] { d.impl().scale_add(a, x.impl(), 0.0, x.impl()); }, "VecScaleAssign");
}
inline void VecScaleAdd(UG4GBVector &d, double a, const UG4GBVector &x, double b, const UG4GBVector &y)
{
    ug4gb_glue::guarded([&] { d.impl().scale_add(a, x.impl(), b, y.impl()); }, "VecScaleAdd");
}
inline void VecScaleAdd(UG4GBVector &d, double a, const UG4GBVector &x, double b, const UG4GBVector &y, double c,
                        const UG4GBVector &z)
{
    ug4gb_glue::guarded(
        [&] {
            d.impl().scale_add(a, x.impl(), b, y.impl());
            d.impl().scale_add(1.0, d.impl(), c, z.impl());
        },
        "VecScaleAdd");
}
inline double VecProd(const UG4GBVector &a, const UG4GBVector &b) { return a.dotprod(b); }
inline double VecNormSquared(const UG4GBVector &a)
{
    const double n = a.norm();
    return n * n;
}

}  // namespace ug
