// ug4gb_domain_disc.h -- the library's FV1 discretisation as ugcore's
// IDomainDiscretization<GPUAlgebra>, so that scripts and plugins assemble
// through the usual DomainDiscretization interface with the GPU algebra.
//
// Reference interfaces:
//   IDomainDiscretization / IAssemble / IDomainErrorIndicator
//     (lib_disc/spatial_disc/domain_disc_interface.h:60-420,
//      lib_disc/assemble_interface.h:109-240);
//   the FV1 element disc of the ConvectionDiffusion plugin, whose settings
//     UG4GBConvectionDiffusionFV1 carries (diffusion, velocity, source,
//     upwind; the element matrices are the engine's, k_fv1.cu);
//   DirichletBoundary::add(value, fct, subsets) with value 0
//     (lib_disc/spatial_disc/constraints/dirichlet_boundary/
//      lagrange_dirichlet_boundary.h).
//
// The engine builds its own hierarchy from the approximation space's coarse
// grid (level 0 of the MultiGrid: vertex positions, elements, the vertices,
// edges and faces of the Dirichlet subsets) refined as often as the
// MultiGrid is (ug4gb_grid_create_unstructured), and numbers its vertices
// its own way.  ugcore numbers the surface DoFs in its DoFDistribution; the
// two numberings are matched once by vertex position
// (ug4gb_perm_from_positions) and every operator and vector crosses the
// boundary through that permutation (ug4gb_perm_matrix / ug4gb_perm_vector):
// the matrices and vectors this class fills are in ugcore's numbering, the
// engine's level operators stay in its own.
//
// Supported: one scalar function ("c"), triangles, quadrilaterals,
// tetrahedra or hexahedra (one type per grid), regular refinement,
// the surface level (GridLevel() / the top level), the stationary
// operator and the two-point time-discrete forms ThetaTimeStep produces
// (mass scalings (1, -1)).  Anything else throws.
//
// Needs ugcore's ugbase on the include path (the header is compiled against
// it where the ugcore tree is present).
#pragma once

#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "lib_disc/function_spaces/approximation_space.h"
#include "lib_disc/spatial_disc/ass_tuner.h"
#include "lib_disc/spatial_disc/domain_disc_interface.h"
#include "ug4gb_algebra.h"

namespace ug {

/// Settings of the FV1 convection-diffusion element disc the engine
/// assembles (ConvectionDiffusionFV1 of the ConvectionDiffusion plugin):
/// -div(K grad c) + div(v c) = f with full upwind.
class UG4GBConvectionDiffusionFV1
{
public:
    explicit UG4GBConvectionDiffusionFV1(const char *functions = "c", const char *subsets = "")
        : m_functions(functions ? functions : "c"), m_subsets(subsets ? subsets : "")
    {
    }
    /// elemDisc:set_diffusion(K), constant
    void set_diffusion(number K)
    {
        m_coef = COEF_CONST;
        m_K = K;
    }
    /// K = exp(factor * amp * sum_m cos(k_m . x + phase_m)) at element
    /// centroids (LognormalRandomField::eval_K form,
    /// lib_disc/spatial_disc/user_data/common_user_data/lognormal_random_field_impl.h)
    void set_diffusion_fourier(const std::vector<number> &k, const std::vector<number> &phase, number amp,
                               number factor)
    {
        m_coef = COEF_FOURIER;
        m_kk = k;
        m_kphase = phase;
        m_kamp = amp;
        m_kfactor = factor;
    }
    /// K = exp(m_e) per element of the surface level (engine element order)
    void set_log_diffusion_elements(const std::vector<number> &m)
    {
        m_coef = COEF_LOG;
        m_logk = m;
    }
    /// v(x) = scale * sum_m -sin(k_m . x + phase_m) c_m (3D curl field)
    void set_velocity_fourier(const std::vector<number> &k, const std::vector<number> &c,
                              const std::vector<number> &phase, number scale)
    {
        m_vk = k;
        m_vc = c;
        m_vphase = phase;
        m_vscale = scale;
    }
    /// elemDisc:set_velocity({vx, vy, vz}): a constant field
    void set_velocity(const std::vector<number> &v)
    {
        UG_COND_THROW(v.size() != 3, "UG4GBConvectionDiffusionFV1: set_velocity needs 3 components");
        // one mode with k = 0 and phase -pi/2: -sin(-pi/2) = 1
        m_vk.assign(3, 0.0);
        m_vc = v;
        m_vphase.assign(1, -1.5707963267948966);
        m_vscale = 1.0;
    }
    /// elemDisc:set_upwind(FullUpwind()) / NoUpwind: "full" or "no"
    void set_upwind(const std::string &type)
    {
        UG_COND_THROW(type != "full" && type != "no", "UG4GBConvectionDiffusionFV1: upwind 'full' or 'no'");
        m_upwind = (type == "full");
    }
    /// elemDisc:set_source(f), constant
    void set_source(number f)
    {
        m_src = SRC_CONST;
        m_f = f;
    }
    /// source f_i = 2 u(seed, i) - 1 (seeded uniform, engine vertex order)
    void set_source_uniform(uint64_t seed)
    {
        m_src = SRC_SEED;
        m_seed = seed;
    }

    /// transfers the settings to the engine discretisation d (nv_top vertices)
    void apply_to(ug4gb_disc *d, int nv_top, ug4gb_ctx *ctx) const
    {
        switch (m_coef) {
            case COEF_CONST: ug4gb::check(ug4gb_disc_set_diffusion_constant(d, m_K), ctx, "diffusion"); break;
            case COEF_FOURIER:
                ug4gb::check(ug4gb_disc_set_diffusion_fourier(d, (int)m_kphase.size(), m_kk.data(), m_kphase.data(),
                                                             m_kamp, m_kfactor),
                             ctx, "diffusion field");
                break;
            case COEF_LOG:
                ug4gb::check(ug4gb_disc_set_log_diffusion_elements(d, m_logk.data()), ctx, "log diffusion");
                break;
        }
        if (!m_vphase.empty()) {
            ug4gb::check(ug4gb_disc_set_velocity_fourier_curl(d, (int)m_vphase.size(), m_vk.data(), m_vc.data(),
                                                             m_vphase.data(), m_vscale),
                         ctx, "velocity");
        }
        ug4gb::check(ug4gb_disc_set_upwind(d, m_upwind ? UG4GB_UPWIND_FULL : UG4GB_UPWIND_NONE), ctx, "upwind");
        if (m_src == SRC_SEED) {
            ug4gb::check(ug4gb_disc_set_source_uniform(d, m_seed), ctx, "source");
        } else {
            std::vector<double> f((size_t)nv_top, m_src == SRC_CONST ? m_f : 0.0);
            ug4gb::check(ug4gb_disc_set_source_vertices(d, f.data()), ctx, "source");
        }
    }
    const std::string &functions() const { return m_functions; }

private:
    enum { COEF_CONST, COEF_FOURIER, COEF_LOG };
    enum { SRC_NONE, SRC_CONST, SRC_SEED };
    std::string m_functions, m_subsets;
    int m_coef = COEF_CONST;
    number m_K = 1.0;
    std::vector<number> m_kk, m_kphase, m_logk;
    number m_kamp = 1.0, m_kfactor = 1.0;
    std::vector<number> m_vk, m_vc, m_vphase;
    number m_vscale = 1.0;
    bool m_upwind = false;
    int m_src = SRC_NONE;
    number m_f = 0.0;
    uint64_t m_seed = 0;
};

template <typename TDomain>
class UG4GBDomainDiscretization : public IDomainDiscretization<GPUAlgebra>
{
public:
    typedef GPUAlgebra algebra_type;
    typedef UG4GBSparseMatrix matrix_type;
    typedef UG4GBVector vector_type;
    typedef typename IDomainErrorIndicator<GPUAlgebra>::error_vector_type error_vector_type;
    static const int dim = TDomain::dim;

    explicit UG4GBDomainDiscretization(SmartPtr<ApproximationSpace<TDomain> > approxSpace)
        : m_spApprox(approxSpace), m_spAssTuner(new AssemblingTuner<GPUAlgebra>)
    {
        UG_COND_THROW(approxSpace.invalid(), "UG4GBDomainDiscretization: no approximation space");
    }

    virtual ~UG4GBDomainDiscretization()
    {
        if (m_td) ug4gb_timedisc_destroy(m_td);
        if (m_perm) ug4gb_perm_destroy(m_perm);
        if (m_disc) ug4gb_disc_destroy(m_disc);
        if (m_grid) ug4gb_grid_destroy(m_grid);
    }

    /// domainDisc:add(elemDisc)
    void add(SmartPtr<UG4GBConvectionDiffusionFV1> elem)
    {
        m_spElem = elem;
        m_dirty = true;
    }
    /// domainDisc:add(dirichletBnd) with dirichletBnd:add(0, "c", subsets):
    /// zero Dirichlet values on these subsets (comma-separated names)
    void add_dirichlet(const char *subsets)
    {
        if (!m_dirichlet.empty()) m_dirichlet += ",";
        m_dirichlet += subsets ? subsets : "";
        m_grid_ready = false;
    }

    /// the engine discretisation and the DoF permutation (for the GPU
    /// multigrid built on the same hierarchy)
    ug4gb_disc *engine_disc()
    {
        ensure_engine();
        return m_disc;
    }
    ug4gb_perm *engine_perm()
    {
        ensure_engine();
        return m_perm;
    }
    int engine_top_level() const { return m_top; }

    // ----------------------------------------------------------- IAssemble
    virtual void assemble_jacobian(matrix_type &J, const vector_type &u, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                ug4gb::check(ug4gb_disc_assemble_jacobian(m_disc, m_top, m_A->get()), ctx(), "assemble_jacobian");
                ug4gb::check(ug4gb_perm_matrix(m_perm, 1, m_A->get(), J.impl().get()), ctx(), "permute jacobian");
            },
            "UG4GBDomainDiscretization::assemble_jacobian");
    }
    virtual void assemble_jacobian(matrix_type &J, const vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_jacobian(J, u, dd->grid_level());
    }
    virtual void assemble_defect(vector_type &d, const vector_type &u, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                ug4gb::check(ug4gb_perm_vector(m_perm, 0, u.impl().get(), m_u->get()), ctx(), "permute u");
                ug4gb::check(ug4gb_disc_assemble_defect(m_disc, m_top, m_u->get(), m_b->get()), ctx(), "defect");
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_b->get(), d.impl().get()), ctx(), "permute defect");
            },
            "UG4GBDomainDiscretization::assemble_defect");
    }
    virtual void assemble_defect(vector_type &d, const vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_defect(d, u, dd->grid_level());
    }
    virtual void assemble_linear(matrix_type &A, vector_type &b, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                ug4gb::check(ug4gb_disc_assemble_linear(m_disc, m_top, m_A->get(), m_b->get()), ctx(), "assemble");
                ug4gb::check(ug4gb_perm_matrix(m_perm, 1, m_A->get(), A.impl().get()), ctx(), "permute matrix");
                b.resize(m_n);
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_b->get(), b.impl().get()), ctx(), "permute rhs");
            },
            "UG4GBDomainDiscretization::assemble_linear");
    }
    virtual void assemble_linear(matrix_type &A, vector_type &b, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_linear(A, b, dd->grid_level());
    }
    virtual void assemble_rhs(vector_type &rhs, const vector_type &u, const GridLevel &gl) { assemble_rhs(rhs, gl); }
    virtual void assemble_rhs(vector_type &rhs, const vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_rhs(rhs, dd->grid_level());
    }
    virtual void assemble_rhs(vector_type &b, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                ug4gb::check(ug4gb_disc_assemble_linear(m_disc, m_top, m_A->get(), m_b->get()), ctx(), "assemble");
                b.resize(m_n);
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_b->get(), b.impl().get()), ctx(), "permute rhs");
            },
            "UG4GBDomainDiscretization::assemble_rhs");
    }
    virtual void assemble_rhs(vector_type &b, ConstSmartPtr<DoFDistribution> dd) { assemble_rhs(b, dd->grid_level()); }
    virtual void adjust_solution(vector_type &u, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                ug4gb::check(ug4gb_perm_vector(m_perm, 0, u.impl().get(), m_u->get()), ctx(), "permute u");
                ug4gb::check(ug4gb_disc_adjust_solution(m_disc, m_top, m_u->get()), ctx(), "adjust");
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_u->get(), u.impl().get()), ctx(), "permute u");
            },
            "UG4GBDomainDiscretization::adjust_solution");
    }
    virtual void adjust_solution(vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        adjust_solution(u, dd->grid_level());
    }
    virtual void assemble_mass_matrix(matrix_type &M, const vector_type &u, const GridLevel &gl)
    {
        // M = (M + 1 * A) - A: the lumped FV1 mass of the time discretisation
        UG_THROW("UG4GBDomainDiscretization: assemble_mass_matrix is assembled through ThetaTimeStep");
    }
    virtual void assemble_mass_matrix(matrix_type &M, const vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_mass_matrix(M, u, dd->grid_level());
    }
    virtual void assemble_stiffness_matrix(matrix_type &A, const vector_type &u, const GridLevel &gl)
    {
        assemble_jacobian(A, u, gl);
    }
    virtual void assemble_stiffness_matrix(matrix_type &A, const vector_type &u, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_jacobian(A, u, dd->grid_level());
    }
    virtual SmartPtr<AssemblingTuner<GPUAlgebra> > ass_tuner() { return m_spAssTuner; }
    virtual ConstSmartPtr<AssemblingTuner<GPUAlgebra> > ass_tuner() const { return m_spAssTuner; }
    virtual size_t num_constraints() const { return 0; }
    virtual SmartPtr<IConstraint<GPUAlgebra> > constraint(size_t i)
    {
        UG_THROW("UG4GBDomainDiscretization: the Dirichlet boundary is part of the engine discretisation");
    }

    // --------------------------------------------- time-dependent forms
    // ThetaTimeStep scalings (theta_time_step.h:230-246): s_m = (1, -1),
    // s_a = (theta dt, (1 - theta) dt); the engine's time discretisation takes
    // theta and dt
    virtual void prepare_timestep(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, number future_time,
                                  ConstSmartPtr<DoFDistribution> dd)
    {
        m_future_time = future_time;
    }
    virtual void prepare_timestep(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, number future_time,
                                  const GridLevel &gl)
    {
        m_future_time = future_time;
    }
    virtual void prepare_timestep_elem(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                       ConstSmartPtr<DoFDistribution> dd)
    {
    }
    virtual void prepare_timestep_elem(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, const GridLevel &gl) {}
    virtual void assemble_jacobian(matrix_type &J, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                   const number s_a, const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                // M + s_a A = the jacobian of a step with theta = 1, dt = s_a
                time_disc(1.0, s_a, vSol);
                ug4gb::check(ug4gb_timedisc_assemble_jacobian(m_td, m_top, m_A->get()), ctx(), "jacobian");
                ug4gb::check(ug4gb_perm_matrix(m_perm, 1, m_A->get(), J.impl().get()), ctx(), "permute");
            },
            "UG4GBDomainDiscretization::assemble_jacobian (time-discrete)");
    }
    virtual void assemble_jacobian(matrix_type &J, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                   const number s_a0, ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_jacobian(J, vSol, s_a0, dd->grid_level());
    }
    virtual void assemble_defect(vector_type &d, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                 const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                                 const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                theta_from_scales(vScaleMass, vScaleStiff, vSol);
                ug4gb::check(ug4gb_perm_vector(m_perm, 0, vSol->solution(0)->impl().get(), m_u->get()), ctx(),
                             "permute u");
                ug4gb::check(ug4gb_timedisc_assemble_defect(m_td, m_top, m_u->get(), m_b->get()), ctx(), "defect");
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_b->get(), d.impl().get()), ctx(), "permute defect");
            },
            "UG4GBDomainDiscretization::assemble_defect (time-discrete)");
    }
    virtual void assemble_defect(vector_type &d, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                 const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                                 ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_defect(d, vSol, vScaleMass, vScaleStiff, dd->grid_level());
    }
    virtual void assemble_linear(matrix_type &A, vector_type &b, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                 const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                                 const GridLevel &gl)
    {
        check_level(gl);
        ensure_engine();
        ug4gb_glue::guarded(
            [&] {
                theta_from_scales(vScaleMass, vScaleStiff, vSol);
                ug4gb::check(ug4gb_timedisc_assemble_linear(m_td, m_top, m_A->get(), m_b->get()), ctx(), "assemble");
                ug4gb::check(ug4gb_perm_matrix(m_perm, 1, m_A->get(), A.impl().get()), ctx(), "permute matrix");
                b.resize(m_n);
                ug4gb::check(ug4gb_perm_vector(m_perm, 1, m_b->get(), b.impl().get()), ctx(), "permute rhs");
            },
            "UG4GBDomainDiscretization::assemble_linear (time-discrete)");
    }
    virtual void assemble_linear(matrix_type &A, vector_type &b, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                 const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                                 ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_linear(A, b, vSol, vScaleMass, vScaleStiff, dd->grid_level());
    }
    virtual void assemble_rhs(vector_type &b, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                              const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                              const GridLevel &gl)
    {
        matrix_type A;
        assemble_linear(A, b, vSol, vScaleMass, vScaleStiff, gl);
    }
    virtual void assemble_rhs(vector_type &b, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                              const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                              ConstSmartPtr<DoFDistribution> dd)
    {
        assemble_rhs(b, vSol, vScaleMass, vScaleStiff, dd->grid_level());
    }
    virtual void adjust_solution(vector_type &u, number time, const GridLevel &gl) { adjust_solution(u, gl); }
    virtual void adjust_solution(vector_type &u, number time, ConstSmartPtr<DoFDistribution> dd)
    {
        adjust_solution(u, dd->grid_level());
    }
    virtual void finish_timestep(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, ConstSmartPtr<DoFDistribution> dd)
    {
    }
    virtual void finish_timestep(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, const GridLevel &gl) {}
    virtual void finish_timestep_elem(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, const GridLevel &gl) {}
    virtual void finish_timestep_elem(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol,
                                      ConstSmartPtr<DoFDistribution> dd)
    {
    }

    // ---------------------------------------------- IDomainErrorIndicator
    virtual void calc_error(const vector_type &u, const GridLevel &gl, error_vector_type *u_vtk = NULL)
    {
        UG_THROW("UG4GBDomainDiscretization: no error estimator (adaptivity is out of scope)");
    }
    virtual void calc_error(const vector_type &u, ConstSmartPtr<DoFDistribution> dd, error_vector_type *u_vtk = NULL)
    {
        calc_error(u, dd->grid_level(), u_vtk);
    }
    virtual void calc_error(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, ConstSmartPtr<DoFDistribution> dd,
                            const std::vector<number> &vScaleMass, const std::vector<number> &vScaleStiff,
                            error_vector_type *u_vtk)
    {
        calc_error(*vSol->solution(0), dd->grid_level(), u_vtk);
    }
    virtual void calc_error(ConstSmartPtr<VectorTimeSeries<vector_type> > vSol, const std::vector<number> &vScaleMass,
                            const std::vector<number> &vScaleStiff, const GridLevel &gl, error_vector_type *u_vtk)
    {
        calc_error(*vSol->solution(0), gl, u_vtk);
    }
    virtual void invalidate_error() {}
    virtual bool is_error_valid() { return false; }

private:
    ug4gb_ctx *ctx() const { return ug4gb_glue::context().get(); }

    void check_level(const GridLevel &gl) const
    {
        UG_COND_THROW(!gl.is_surface() && gl.level() != GridLevel::TOP,
                      "UG4GBDomainDiscretization: only the surface (top) level is assembled here; the GPU "
                      "multigrid assembles its own levels");
    }

    /// the engine's grid, discretisation, buffers and DoF permutation,
    /// built from the approximation space on first use
    void ensure_engine()
    {
        if (!m_grid_ready) build_grid();
        if (m_dirty) {
            UG_COND_THROW(m_spElem.invalid(), "UG4GBDomainDiscretization: no element discretisation added");
            ug4gb_glue::guarded([&] { m_spElem->apply_to(m_disc, m_n, ctx()); }, "UG4GBDomainDiscretization");
            m_dirty = false;
        }
    }

    void build_grid()
    {
        SmartPtr<TDomain> dom = m_spApprox->domain();
        MultiGrid &mg = *dom->grid();
        typename TDomain::position_accessor_type &aaPos = dom->position_accessor();
        ISubsetHandler &sh = *dom->subset_handler();
        // Dirichlet subsets by name
        std::vector<int> dsub;
        {
            std::string s = m_dirichlet;
            size_t a = 0;
            while (a <= s.size()) {
                size_t b = s.find(',', a);
                if (b == std::string::npos) b = s.size();
                std::string nm = s.substr(a, b - a);
                while (!nm.empty() && nm.front() == ' ') nm.erase(nm.begin());
                while (!nm.empty() && nm.back() == ' ') nm.pop_back();
                if (!nm.empty()) {
                    const int si = sh.get_subset_index(nm.c_str());
                    UG_COND_THROW(si < 0, "UG4GBDomainDiscretization: no subset '" << nm << "'");
                    dsub.push_back(si);
                }
                a = b + 1;
            }
        }
        auto in_dirichlet = [&](GridObject *o) {
            const int si = sh.get_subset_index(o);
            for (int d : dsub)
                if (d == si) return true;
            return false;
        };
        // coarse vertices
        std::vector<double> coords;
        std::vector<unsigned char> dv;
        std::map<Vertex *, int> vid;
        for (VertexIterator it = mg.begin<Vertex>(0); it != mg.end<Vertex>(0); ++it) {
            vid[*it] = (int)vid.size();
            for (int d = 0; d < dim; ++d) coords.push_back(aaPos[*it][d]);
            dv.push_back(in_dirichlet(*it) ? 1 : 0);
        }
        // coarse elements of the top dimension, one type
        int et = -1;
        std::vector<int> elems;
        auto take = [&](auto *tag, int type) {
            typedef typename std::remove_pointer<decltype(tag)>::type TElem;
            if (mg.template num<TElem>(0) == 0) return;
            UG_COND_THROW(et >= 0, "UG4GBDomainDiscretization: one element type per grid");
            et = type;
            for (typename geometry_traits<TElem>::iterator it = mg.template begin<TElem>(0);
                 it != mg.template end<TElem>(0); ++it)
                for (size_t i = 0; i < (*it)->num_vertices(); ++i) elems.push_back(vid[(*it)->vertex(i)]);
        };
        if (dim == 2) {
            take((Triangle *)nullptr, UG4GB_TRI);
            take((Quadrilateral *)nullptr, UG4GB_QUAD);
        } else {
            take((Tetrahedron *)nullptr, UG4GB_TET);
            take((Hexahedron *)nullptr, UG4GB_HEX);
        }
        UG_COND_THROW(et < 0, "UG4GBDomainDiscretization: no triangles, quadrilaterals, tetrahedra or hexahedra");
        // Dirichlet edges and faces of the coarse grid (the refinement
        // carries their subsets to the new vertices)
        std::vector<int> dedges, dfaces;
        for (EdgeIterator it = mg.begin<Edge>(0); it != mg.end<Edge>(0); ++it)
            if (in_dirichlet(*it)) {
                dedges.push_back(vid[(*it)->vertex(0)]);
                dedges.push_back(vid[(*it)->vertex(1)]);
            }
        if (dim == 3)
            for (FaceIterator it = mg.begin<Face>(0); it != mg.end<Face>(0); ++it)
                if (in_dirichlet(*it)) {
                    for (size_t i = 0; i < 4; ++i)
                        dfaces.push_back(i < (*it)->num_vertices() ? vid[(*it)->vertex(i)] : -1);
                }
        const int nref = (int)mg.num_levels() - 1;
        // surface DoF positions in ugcore's numbering
        ConstSmartPtr<DoFDistribution> dd = m_spApprox->dof_distribution(GridLevel());
        const size_t n = dd->num_indices();
        std::vector<double> pos(n * dim, 0.0);
        std::vector<size_t> ind;
        for (typename DoFDistribution::traits<Vertex>::const_iterator it = dd->begin<Vertex>();
             it != dd->end<Vertex>(); ++it) {
            dd->inner_algebra_indices(*it, ind);
            for (size_t k : ind)
                for (int d = 0; d < dim; ++d) pos[k * dim + d] = aaPos[*it][d];
        }
        ug4gb_glue::guarded(
            [&] {
                ug4gb_ctx *c = ctx();
                ug4gb_grid *g = nullptr;
                ug4gb::check(ug4gb_grid_create_unstructured(c, et, (int)vid.size(), coords.data(),
                                                            (int)(elems.size() / (et == UG4GB_HEX ? 8 : (et == UG4GB_TRI ? 3 : 4))),
                                                            elems.data(), dv.data(), (int)(dedges.size() / 2),
                                                            dedges.empty() ? nullptr : dedges.data(),
                                                            (int)(dfaces.size() / 4),
                                                            dfaces.empty() ? nullptr : dfaces.data(), nref, &g),
                             c, "engine grid");
                if (m_td) ug4gb_timedisc_destroy(m_td);
                if (m_perm) ug4gb_perm_destroy(m_perm);
                if (m_disc) ug4gb_disc_destroy(m_disc);
                if (m_grid) ug4gb_grid_destroy(m_grid);
                m_td = nullptr;
                m_perm = nullptr;
                m_grid = g;
                m_top = ug4gb_grid_num_levels(g) - 1;
                int nv = 0, ne = 0, k = 0, d = 0;
                ug4gb::check(ug4gb_grid_level_info(g, m_top, &nv, &ne, &k, &d), c, "level info");
                UG_COND_THROW((size_t)nv != n, "UG4GBDomainDiscretization: the engine's top level has "
                                                   << nv << " vertices, the DoF distribution " << n);
                ug4gb::check(ug4gb_perm_from_positions(c, g, m_top, (int)n, pos.data(), 1e-9, &m_perm), c,
                             "DoF permutation");
                ug4gb::check(ug4gb_disc_create(c, g, &m_disc), c, "engine disc");
                m_n = (int)n;
                m_A.reset(new ug4gb::Matrix(c));
                m_b.reset(new ug4gb::Vector(c, m_n));
                m_u.reset(new ug4gb::Vector(c, m_n));
            },
            "UG4GBDomainDiscretization: engine set-up");
        m_grid_ready = true;
        m_dirty = true;
    }

    // the engine's theta step from ugcore's two-point scalings
    void theta_from_scales(const std::vector<number> &sm, const std::vector<number> &sa,
                           ConstSmartPtr<VectorTimeSeries<vector_type> > vSol)
    {
        UG_COND_THROW(sm.size() != 2 || sa.size() != 2 || sm[0] != 1.0 || sm[1] != -1.0,
                      "UG4GBDomainDiscretization: two time points with mass scalings (1, -1) only");
        const number dt = sa[0] + sa[1];
        UG_COND_THROW(!(dt > 0.0), "UG4GBDomainDiscretization: non-positive time step");
        time_disc(sa[0] / dt, dt, vSol);
    }

    void time_disc(number theta, number dt, ConstSmartPtr<VectorTimeSeries<vector_type> > vSol)
    {
        ug4gb_ctx *c = ctx();
        if (!m_td) ug4gb::check(ug4gb_timedisc_create(c, m_disc, &m_td), c, "time disc");
        ug4gb::check(ug4gb_timedisc_set_theta(m_td, theta), c, "theta");
        // the previous solution (time point 1 of the series) in engine order
        const int old = vSol->size() > 1 ? 1 : 0;
        ug4gb::check(ug4gb_perm_vector(m_perm, 0, vSol->solution(old)->impl().get(), m_u->get()), c, "permute");
        ug4gb::check(ug4gb_timedisc_prepare_step(m_td, m_u->get(), vSol->time(old), dt), c, "prepare step");
    }

    SmartPtr<ApproximationSpace<TDomain> > m_spApprox;
    SmartPtr<AssemblingTuner<GPUAlgebra> > m_spAssTuner;
    SmartPtr<UG4GBConvectionDiffusionFV1> m_spElem;
    std::string m_dirichlet;
    bool m_grid_ready = false, m_dirty = true;
    ug4gb_grid *m_grid = nullptr;
    ug4gb_disc *m_disc = nullptr;
    ug4gb_perm *m_perm = nullptr;
    ug4gb_timedisc *m_td = nullptr;
    int m_top = 0, m_n = 0;
    number m_future_time = 0.0;
    std::unique_ptr<ug4gb::Matrix> m_A;
    std::unique_ptr<ug4gb::Vector> m_b, m_u;
};

}  // namespace ug
