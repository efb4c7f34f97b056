// ug4gb_preconditioner.h -- the library's geometric multigrid as a ugcore
// ILinearIterator of the GPU algebra, for ugcore's own Krylov solvers.
//
// ugcore's CG / BiCGStab (lib_algebra/operator/linear_solver/cg.h:103-230,
// bicgstab.h:112-400) call their preconditioner through ILinearIterator
// (lib_algebra/operator/interface/linear_iterator.h:80-170): init(J) with the
// operator, then apply(c, d) once per step.  UG4GBGeometricMultiGrid takes the
// operator's matrix from the MatrixOperator<UG4GBSparseMatrix, UG4GBVector>
// the solver is initialised with, sets the library's multigrid up with it
// (AssembledMultiGridCycle::init, mg_solver_impl.hpp:380) and applies one
// cycle per call on the device.  The bridge registers it as the "GPU1"
// GeometricMultiGrid.
//
// Needs ugcore's lib_algebra headers on the include path, like ug4gb_algebra.h.
#pragma once

#include <memory>
#include <string>

#include "lib_algebra/operator/interface/linear_iterator.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "ug4gb_algebra.h"

namespace ug {

class UG4GBGeometricMultiGrid : public ILinearIterator<UG4GBVector>
{
public:
    typedef UG4GBVector vector_type;
    typedef UG4GBSparseMatrix matrix_type;
    typedef MatrixOperator<matrix_type, vector_type> matrix_operator_type;
    typedef ILinearIterator<vector_type> base_type;

    /// disc: the library discretisation of the grid hierarchy the levels come from
    explicit UG4GBGeometricMultiGrid(ug4gb_disc *disc) : m_disc(disc) { create(); }
    /// the multigrid of a UG4GBDomainDiscretization (ug4gb_domain_disc.h):
    /// operators and vectors come in ugcore's DoF numbering and cross to the
    /// engine's through the discretisation's DoF permutation
    template <class TDomainDisc>
    explicit UG4GBGeometricMultiGrid(SmartPtr<TDomainDisc> domainDisc)
        : m_keep(domainDisc), m_disc(domainDisc->engine_disc()), m_perm(domainDisc->engine_perm())
    {
        create();
    }
    UG4GBGeometricMultiGrid(const UG4GBGeometricMultiGrid &o)
        : base_type(o), m_keep(o.m_keep), m_disc(o.m_disc), m_perm(o.m_perm), m_cfg(o.m_cfg)
    {
        create();
    }

    /// Jacobi (UG4GB_SMOOTHER_JACOBI, damp 0.6 as Jacobi(0.6)), or the
    /// multicolour Gauss-Seidel / symmetric Gauss-Seidel / ILU variants
    void set_smoother(int kind, double damp)
    {
        m_cfg.smoother = m_cfg.smoother2 = kind;
        m_cfg.damp = m_cfg.damp2 = damp;
        configure();
    }
    /// set_presmoother / set_postsmoother (mg_solver.h:179-183): damp is the
    /// Jacobi damping, the SOR relaxation of the Gauss-Seidel kinds
    /// (including UG4GB_SMOOTHER_MCBGS, backward) or the ILU factor
    void set_presmoother(int kind, double damp)
    {
        m_cfg.smoother = kind;
        m_cfg.damp = damp;
        configure();
    }
    void set_postsmoother(int kind, double damp)
    {
        m_cfg.smoother2 = kind;
        m_cfg.damp2 = damp;
        configure();
    }
    void set_cycle_type(int c) { m_cfg.cycle = c; configure(); }
    void set_num_presmooth(int n) { m_cfg.nu1 = n; configure(); }
    void set_num_postsmooth(int n) { m_cfg.nu2 = n; configure(); }
    void set_base_level(int l) { m_cfg.base = l; configure(); }
    /// "fp64" or "mixed" (FP32 multigrid)
    void set_precision(const std::string &p)
    {
        m_cfg.precision = (p == "mixed") ? UG4GB_PREC_MIXED : UG4GB_PREC_FP64;
        configure();
    }
    void set_rap(bool rap) { m_cfg.rap = rap; configure(); }
    /// AssembledMultiGridCycle::set_transfer with a StdTransfer's damping
    /// (std_transfer.h:92,95)
    void set_transfer_damping(double prolongation, double restriction)
    {
        ug4gb_glue::guarded(
            [&] {
                ug4gb_ctx *ctx = ug4gb_glue::context().get();
                ug4gb::check(ug4gb_gmg_set_prolongation_damping(m_gmg, prolongation), ctx, "prolongation damping");
                ug4gb::check(ug4gb_gmg_set_restriction_damping(m_gmg, restriction), ctx, "restriction damping");
            },
            "GPU GeometricMultiGrid::set_transfer");
    }
    /// coarse levels assembled as a time discretisation's jacobian (null: stationary)
    void set_discretization(ug4gb_timedisc *td)
    {
        ug4gb_glue::guarded(
            [&] { ug4gb::check(ug4gb_gmg_set_time_disc(m_gmg, td), ug4gb_glue::context().get(), "time disc"); },
            "GPU GeometricMultiGrid::set_discretization");
    }

    virtual const char *name() const { return "GPU GeometricMultiGrid"; }
    virtual bool supports_parallel() const { return false; }

    virtual bool init(SmartPtr<ILinearOperator<vector_type> > J, const vector_type &u) { return init(J); }
    virtual bool init(SmartPtr<ILinearOperator<vector_type> > L)
    {
        SmartPtr<matrix_operator_type> op = L.template cast_dynamic<matrix_operator_type>();
        if (op.invalid()) UG_THROW("GPU GeometricMultiGrid: the operator is not an assembled GPU matrix");
        m_A = &op->get_matrix();
        ug4gb_glue::guarded(
            [&] {
                ug4gb_ctx *ctx = ug4gb_glue::context().get();
                const ug4gb_matrix *A = m_A->impl().get();
                if (m_perm) {
                    // the top operator in the engine's numbering
                    if (!m_Aeng) m_Aeng.reset(new ug4gb::Matrix(ctx));
                    ug4gb::check(ug4gb_perm_matrix(m_perm, 0, A, m_Aeng->get()), ctx, "permute operator");
                    A = m_Aeng->get();
                    const int n = (int)m_A->num_rows();
                    if (!m_deng || m_deng->size() != n) {
                        m_deng.reset(new ug4gb::Vector(ctx, n));
                        m_ceng.reset(new ug4gb::Vector(ctx, n));
                    }
                }
                ug4gb::check(ug4gb_gmg_init(m_gmg, A), ctx, "gmg init");
            },
            "GPU GeometricMultiGrid::init");
        return true;
    }

    /// c = M d (one multigrid cycle from c = 0)
    virtual bool apply(vector_type &c, const vector_type &d)
    {
        ug4gb_glue::guarded(
            [&] {
                ug4gb_ctx *ctx = ug4gb_glue::context().get();
                if (m_perm) {
                    ug4gb::check(ug4gb_perm_vector(m_perm, 0, d.impl().get(), m_deng->get()), ctx, "permute d");
                    ug4gb::check(ug4gb_gmg_apply(m_gmg, m_ceng->get(), m_deng->get()), ctx, "gmg apply");
                    ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_ceng->get(), c.impl().get()), ctx, "permute c");
                } else {
                    ug4gb::check(ug4gb_gmg_apply(m_gmg, c.impl().get(), d.impl().get()), ctx, "gmg apply");
                }
            },
            "GPU GeometricMultiGrid::apply");
        return true;
    }

    /// c = M d, then d -= A c
    virtual bool apply_update_defect(vector_type &c, vector_type &d)
    {
        if (!m_A) UG_THROW("GPU GeometricMultiGrid: apply_update_defect before init");
        apply(c, d);
        m_A->matmul_minus(d, c);
        return true;
    }

    virtual SmartPtr<base_type> clone() { return make_sp(new UG4GBGeometricMultiGrid(*this)); }

    virtual ~UG4GBGeometricMultiGrid()
    {
        if (m_gmg) ug4gb_gmg_destroy(m_gmg);
    }

private:
    struct Config {
        int smoother = UG4GB_SMOOTHER_JACOBI, smoother2 = UG4GB_SMOOTHER_JACOBI;
        double damp = 0.6, damp2 = 0.6;
        int cycle = 1, nu1 = 2, nu2 = 2, base = 0;
        int precision = UG4GB_PREC_FP64;
        bool rap = false;
    };

    void create()
    {
        ug4gb_glue::guarded(
            [&] { ug4gb::check(ug4gb_gmg_create(ug4gb_glue::context().get(), m_disc, &m_gmg), nullptr, "gmg"); },
            "GPU GeometricMultiGrid");
        configure();
    }

    void configure()
    {
        ug4gb_glue::guarded(
            [&] {
                ug4gb_ctx *ctx = ug4gb_glue::context().get();
                ug4gb::check(ug4gb_gmg_set_presmoother(m_gmg, m_cfg.smoother, m_cfg.damp), ctx, "presmoother");
                ug4gb::check(ug4gb_gmg_set_postsmoother(m_gmg, m_cfg.smoother2, m_cfg.damp2), ctx, "postsmoother");
                ug4gb::check(ug4gb_gmg_set_cycle_type(m_gmg, m_cfg.cycle), ctx, "cycle");
                ug4gb::check(ug4gb_gmg_set_num_presmooth(m_gmg, m_cfg.nu1), ctx, "presmooth");
                ug4gb::check(ug4gb_gmg_set_num_postsmooth(m_gmg, m_cfg.nu2), ctx, "postsmooth");
                ug4gb::check(ug4gb_gmg_set_base_level(m_gmg, m_cfg.base), ctx, "base level");
                ug4gb::check(ug4gb_gmg_set_precision(m_gmg, m_cfg.precision), ctx, "precision");
                ug4gb::check(ug4gb_gmg_set_rap(m_gmg, m_cfg.rap ? 1 : 0), ctx, "rap");
            },
            "GPU GeometricMultiGrid configuration");
    }

    SmartPtr<void> m_keep;               // the domain discretisation that owns m_disc / m_perm, or null
    ug4gb_disc *m_disc = nullptr;
    ug4gb_perm *m_perm = nullptr;
    ug4gb_gmg *m_gmg = nullptr;
    Config m_cfg;
    const matrix_type *m_A = nullptr;
    std::shared_ptr<ug4gb::Matrix> m_Aeng;   // the top operator in the engine's numbering
    std::shared_ptr<ug4gb::Vector> m_deng, m_ceng;
};

}  // namespace ug
