// disc.cuh -- launch interface of the FV1 assembly / coefficient / gradient
// kernels (k_fv1.cu) used by the host orchestration.
#pragma once

#include <vector>

#include "common.cuh"

namespace ug4gb {

struct AsmArgs {
    const double *coords;
    const int *elems;
    int ne;
    const double *K;          // per element
    const double *f;          // per vertex or null
    uint64_t f_seed;          // seeded uniform source when use_seed
    int use_seed;
    int vmodes;               // velocity field (3D curl form), 0 = none
    const double *vk, *vc, *vphase;
    double vscale;
    uint64_t vel_version = 0;  // changes with the velocity field (cached fluxes)
    const int *rowptr;        // level CRS to scatter into
    const int *col;
    double *val;
    double *b;                // rhs or null
    int cx, cy, cz;           // structured cell counts (set by the coloured launch)
    const int *elist = nullptr;  // unstructured: elements of the launched colour
    int nlist = 0;
    // instationary assembly (ThetaTimeStep): element matrix sm0 M_e + sa0 A_e
    // with the lumped FV1 mass M_e = diag(|SCV_i|); with b, the rhs of one
    // previous time point: sa0 f_e - sm1 M_e u_old - sa1 A_e u_old + sa1 f_e
    int inst = 0;
    int k_uniform = 0;        // K holds one value for all elements: k_value
    double k_value = 0.0;
    double sm0 = 0.0, sa0 = 1.0, sm1 = 0.0, sa1 = 0.0;
    const double *u_old = nullptr;
    // defect assembly (launch_defect): d += per-element defect of u
    const double *u = nullptr;
    double *d = nullptr;
};

// scalings of a time-discrete assembly (one previous time point)
struct TimeScale {
    double sm0, sa0, sm1, sa1;
    const double *u_old;   // top-level previous solution (device), for the rhs
};

void launch_assemble(Ctx &c, const Level &L, const AsmArgs &a);
// class geometry of a structured level, kept for the row-wise assembly
struct RowAsmCache {
    bool ready = false, usable = false;
    std::vector<double> A, vol;         // unit-coefficient element matrices, SCV volumes per class
    DevBuf<double> normal, ipoff;       // SCVF area normals / ips relative to the cell origin per class
    DevBuf<double> flux;                // per element and SCVF: v(ip).n (convection)
    uint64_t flux_version = 0;          // velocity field version flux holds (0: none)
    double volsum = 0.0;                // sum of an interior vertex's SCV volumes (gather order)
    DevBuf<int> brows;                  // the rows on the box boundary
    int nbrows = 0;
};
// stationary assembly of a structured level row by row (k_fv1_rows.cu):
// every value of A and b written once, Dirichlet rows included; returns
// false, launching nothing, where it does not apply
bool launch_assemble_rows(Ctx &c, const Level &L, const AsmArgs &a, RowAsmCache &cache);
void launch_dirichlet(Ctx &c, const Level &L, Csr &A, double *b);
// d = defect of a.u on level L (a.d must be zero on entry; Dirichlet rows 0);
// stationary, or instationary with a.inst and the scalings of AsmArgs
void launch_defect(Ctx &c, const Level &L, const AsmArgs &a);
// u = 0 at the Dirichlet vertices of L (DirichletBoundary::adjust_solution)
void launch_dirichlet_values(Ctx &c, const Level &L, double *u);
void launch_coef_fourier(Ctx &c, const Level &L, int nmodes, const double *k, const double *phase, double amp,
                         double factor, double *K);
void coarsen_log(Ctx &c, const Level &F, const Level &Cl, const double *logf, double *logc);
// unstructured levels: coarse log K = mean of the element's children
void coarsen_log_children(Ctx &c, const Level &F, const Level &Cl, const double *logf, double *logc);
void exp_elements(Ctx &c, const double *m, int n, double *K);
void launch_grad_logk(Ctx &c, const Level &L, const double *K, const double *u, const double *lam, double *g);
void launch_grad_source(Ctx &c, const Level &L, const double *lam, double *g);

}  // namespace ug4gb
