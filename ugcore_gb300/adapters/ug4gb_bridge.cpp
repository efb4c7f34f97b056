// ug4gb_bridge.cpp -- registers the GPU classes with ugcore's registry, so
// that Lua scripts and plugins reach them by the usual names.
//
// Two ways in, both through ugcore's Registry (registry/registry.h:179-291):
//   - as a plugin: InitUGPlugin_UG4GB(Registry*, std::string), the entry
//     point ugcore's plugin loader calls (common/util/plugin_util_dynamic.cpp:
//     137-148);
//   - from ugcore's bridge (bridge/bridge.cpp) with RegisterUG4GB, where
//     GPUAlgebra is in CompileAlgebraList (bridge/util_algebra_dependent.h:
//     60-62): the algebra-templated classes (CG, BiCGStab, Jacobi, ...) are
//     then registered with the "GPU1" suffix by ugcore itself.
// What this file adds, per domain (suffix 2d / 3d, grouped by tag so that
// InitUG(dim, AlgebraType("GPU", 1)) selects them):
//   DomainDiscretizationGPU     UG4GBDomainDiscretization (ug4gb_domain_disc.h)
//   ConvectionDiffusionFV1GPU   UG4GBConvectionDiffusionFV1 (the element disc's settings)
//   GeometricMultiGridGPU       UG4GBGeometricMultiGrid built on a DomainDiscretizationGPU
// The registration follows the pattern of ugcore's own disc bridges
// (bridge/disc_bridges/multigrid_bridge.cpp:187-220).
#include <string>

#include "bridge/util.h"
#include "bridge/util_domain_dependent.h"
#include "registry/registry.h"
#include "ug4gb_domain_disc.h"
#include "ug4gb_preconditioner.h"

namespace ug {
namespace bridge {
namespace UG4GB {

struct Functionality {
    template <typename TDomain>
    static void Domain(Registry &reg, std::string grp)
    {
        const std::string suffix = GetDomainSuffix<TDomain>();
        const std::string tag = GetDomainTag<TDomain>();
        // the discretisation
        {
            typedef UG4GBDomainDiscretization<TDomain> T;
            typedef IDomainDiscretization<GPUAlgebra> TBase;
            const std::string name = std::string("DomainDiscretizationGPU").append(suffix);
            reg.add_class_<T, TBase>(name, grp)
                .template add_constructor<void (*)(SmartPtr<ApproximationSpace<TDomain> >)>("ApproximationSpace")
                .add_method("add", &T::add, "", "ElemDisc")
                .add_method("add_dirichlet", &T::add_dirichlet, "", "Subsets")
                .set_construct_as_smart_pointer(true);
            reg.add_class_to_group(name, "DomainDiscretizationGPU", tag);
        }
        // its multigrid
        {
            typedef UG4GBGeometricMultiGrid T;
            typedef ILinearIterator<UG4GBVector> TBase;
            const std::string name = std::string("GeometricMultiGridGPU").append(suffix);
            reg.add_class_<T, TBase>(name, grp)
                .template add_constructor<void (*)(SmartPtr<UG4GBDomainDiscretization<TDomain> >)>(
                    "DomainDiscretization")
                .add_method("set_smoother", &T::set_smoother, "", "Kind#Damping")
                .add_method("set_presmoother", &T::set_presmoother, "", "Kind#Damping")
                .add_method("set_postsmoother", &T::set_postsmoother, "", "Kind#Damping")
                .add_method("set_cycle_type", &T::set_cycle_type, "", "Cycle Type")
                .add_method("set_num_presmooth", &T::set_num_presmooth, "", "Number PreSmooth Steps")
                .add_method("set_num_postsmooth", &T::set_num_postsmooth, "", "Number PostSmooth Steps")
                .add_method("set_base_level", &T::set_base_level, "", "Base Level")
                .add_method("set_precision", &T::set_precision, "", "fp64|mixed")
                .add_method("set_rap", &T::set_rap, "", "Galerkin coarse operators")
                .add_method("set_transfer_damping", &T::set_transfer_damping, "", "Prolongation#Restriction")
                .set_construct_as_smart_pointer(true);
            reg.add_class_to_group(name, "GeometricMultiGridGPU", tag);
        }
    }

    static void Common(Registry &reg, std::string grp)
    {
        typedef UG4GBConvectionDiffusionFV1 T;
        reg.add_class_<T>("ConvectionDiffusionFV1GPU", grp)
            .template add_constructor<void (*)(const char *, const char *)>("Functions#Subsets")
            .add_method("set_diffusion", &T::set_diffusion, "", "Diffusion")
            .add_method("set_velocity", &T::set_velocity, "", "Velocity")
            .add_method("set_upwind", &T::set_upwind, "", "full|no")
            .add_method("set_source", &T::set_source, "", "Source")
            .add_method("set_source_uniform", &T::set_source_uniform, "", "Seed")
            .set_construct_as_smart_pointer(true);
    }
};

}  // namespace UG4GB

void RegisterUG4GB(Registry &reg, std::string grp)
{
    grp.append("/UG4GB");
    typedef UG4GB::Functionality Functionality;
    try {
        RegisterCommon<Functionality>(reg, grp);
        RegisterDomainDependent<Functionality>(reg, grp);
    }
    UG_REGISTRY_CATCH_THROW(grp);
}

}  // namespace bridge
}  // namespace ug

extern "C" void InitUGPlugin_UG4GB(ug::bridge::Registry *reg, std::string grp)
{
    ug::bridge::RegisterUG4GB(*reg, grp);
}
