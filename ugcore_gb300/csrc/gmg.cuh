// gmg.cuh -- host-side objects behind the C ABI handles.
#pragma once

#include <memory>

#include "common.cuh"
#include "disc.cuh"
#include "k_solve.cuh"

struct ug4gb_ctx {
    ug4gb::Ctx c;
    int refs = 1;          // the context itself + every live child handle
    bool closed = false;   // ug4gb_destroy called; freed when refs reaches 0
};

// Child handles keep their context alive, so handles may be destroyed in any
// order (e.g. by a garbage collector at interpreter exit).
extern "C" {
void ug4gb_ctx_retain(ug4gb_ctx *ctx);
void ug4gb_ctx_release(ug4gb_ctx *ctx);
}

// process-wide unique id of a grid (never reused, unlike an address after free)
extern "C" uint64_t ug4gb_next_grid_uid();

struct ug4gb_grid {
    ug4gb_ctx *ctx = nullptr;
    int elem_type = 0;
    uint64_t uid = ug4gb_next_grid_uid();
    std::vector<ug4gb::Level> lev;
};

struct ug4gb_vector {
    ug4gb_ctx *ctx = nullptr;
    int n = 0;
    double *d = nullptr;
    ug4gb::DevBuf<double> own;
};

struct ug4gb_matrix {
    ug4gb_ctx *ctx = nullptr;
    ug4gb::Csr A;
    ug4gb::OpMat<double> op;              // solve format of A (SELL-32 or diagonal)
    bool op_valid = false;
    uint64_t pattern_grid = 0;            // uid of the grid (and the level) whose element pattern A holds
    int pattern_level = -1;
    // the transposed element pattern of a level (the adjoint operator), else 0
    uint64_t derived_key = 0;
    // layout of op, valid while the pattern has the key op_key (0: unknown)
    ug4gb::OpLayout op_layout;
    uint64_t op_key = 0;
    // transposition permutation of the adjoint operator and its source key
    ug4gb::DevBuf<int> tperm;
    uint64_t tperm_key = 0;
    // pattern key for which the pattern was found symmetric (in-place adjoint)
    uint64_t sym_key = 0;
    // identity of the current pattern: the element pattern of (grid, level),
    // or the transposed one; 0 = any other (set from arrays, products, ...)
    uint64_t pattern_key() const
    {
        if (pattern_grid) return (pattern_grid << 6) + (uint64_t)(pattern_level + 1);
        return derived_key;
    }
    void ensure_op()
    {
        if (!op_valid) {
            const uint64_t key = pattern_key();
            if (!key || key != op_key) op_layout.known = false;
            ug4gb::op_from_csr_cached<double>(ctx->c, A, op, nullptr, ctx->c.allow_dia, op_layout);
            op_key = key;
            op_valid = true;
        }
    }
};

namespace ug4gb {

enum CoefKind { COEF_CONST = 0, COEF_FOURIER = 1, COEF_LOG_ELEMS = 2 };

struct DiscImpl {
    int coef_kind = COEF_CONST;
    double K_const = 1.0;
    int kmodes = 0;
    DevBuf<double> kk, kphase;
    double kamp = 1.0, kfactor = 1.0;
    DevBuf<double> m_top;                  // COEF_LOG_ELEMS
    std::vector<DevBuf<double>> Klev;      // cache per level
    std::vector<bool> Kvalid;
    int vmodes = 0;
    uint64_t vel_version = 0;              // counts velocity field changes
    DevBuf<double> vk, vc, vphase;
    double vscale = 1.0;
    int upwind = 0;
    DevBuf<double> f_top;
    int f_kind = 0;                        // 0 none, 1 array, 2 seeded uniform
    uint64_t f_seed = 0;
    std::vector<RowAsmCache> rows;         // per level: class geometry of the row-wise assembly
};

template <class V>
struct GLevel {
    int n = 0;
    Csr A;                       // FP64 level operator
    OpMat<V> At;                 // Jacobi: A * diag(dinv); MCGS: A
    DevBuf<V> dinv, dfac;        // Jacobi: dinv = 1/(a_ii/damp), dfac = a_ii/damp; MCGS: relax/a_ii, 1
    DevBuf<V> dinv2;             // Gauss-Seidel post-smoother with its own relaxation: relax2/a_ii
    Csr P, R;                    // P: this x coarse, R: coarse x this (FP64, exportable)
    OpMat<V> Ps, Rs;
    bool grid_transfer = false;  // apply P and R from grid indices (structured hierarchy)
    std::shared_ptr<Sweep2Op> sweep2;   // At prepared for two Jacobi steps per pass (smooth_pair), or null
    GridPair gp{};
    DevBuf<V> sc, dA, dB, w, t;
    V *dcur = nullptr;
    std::vector<DevBuf<int>> crow;   // MCGS / ILU colour row lists
    std::vector<int> ncrow;
    DevBuf<int> vcolor;              // unstructured levels: colours of the operator's own graph
    IluFactors<V> ilu;               // ILU smoother factors
    DevBuf<V> y;                     // ILU forward-substitution scratch
    // kept for a re-init on the same structure (values refreshed in place)
    OpLayout At_lay;                 // layout of At
    bool asm_ok = false;             // A holds this level's pattern (re-assembled in place)
    int sym = -1;                    // A's pattern is symmetric (1), not (0), unknown (-1)
    DevBuf<double> dinv64, dfac64;   // FP64 Jacobi factors
    DevBuf<double> dinv2_64;
};

struct GmgBase {
    virtual ~GmgBase() = default;
    virtual int top() const = 0;
    virtual bool is_fp32() const = 0;
    virtual void *sc_top() = 0;
    // z = M d_top (d_top FP64, device); returns z in FP64.  rho = (z, r_rho)
    // is fused into the last kernel when possible (rho_done tells).
    // top_ready: the caller already wrote d_top in level precision into
    // top_defect_buffer() (mixed precision), so no conversion pass is needed.
    virtual const double *apply(Ctx &c, const double *dtop, const int *skip, const double *r_rho, RedArgs *red,
                                int rho_kind, bool &rho_done, bool top_ready = false) = 0;
    // FP32 buffer a producer of d_top may fill (mixed precision), else null
    virtual float *top_defect_buffer() = 0;
    // a base factorisation done on the device without a wait reports a
    // singular matrix here: called after the caller's stream was synchronised
    virtual void check_base() {}
    virtual const Csr &P(int l) const = 0;
    virtual const Csr &R(int l) const = 0;
    virtual const Csr &levelA(int l) const = 0;   // FP64 operator of level l (re-assembled or R A P)
    virtual int base_level() const = 0;
    // the device buffers the cycle's kernels use: equal signatures before and
    // after a re-init mean the captured graphs stay valid
    virtual uint64_t signature() const = 0;
};

}  // namespace ug4gb

struct ug4gb_disc {
    ug4gb_ctx *ctx = nullptr;
    const ug4gb_grid *g = nullptr;
    ug4gb::DiscImpl d;
};

// ThetaTimeStep (lib_disc/time_disc/theta_time_step.h:165-300): one previous
// time point; scalings s_m = (1, -1), s_a = (theta dt, (1 - theta) dt)
// (update_scaling, theta_time_step.h:230-246)
struct ug4gb_timedisc {
    ug4gb_ctx *ctx = nullptr;
    ug4gb_disc *disc = nullptr;
    double theta = 1.0;
    double dt = 0.0;
    double time = 0.0;           // time of the previous solution; future time = time + dt
    bool prepared = false;
    ug4gb::DevBuf<double> u_old;
    ug4gb::TimeScale scale() const
    {
        return ug4gb::TimeScale{1.0, theta * dt, -1.0, (1.0 - theta) * dt, u_old.p};
    }
    ug4gb::TimeScale jacobian_scale() const
    {
        return ug4gb::TimeScale{1.0, theta * dt, 0.0, 0.0, nullptr};
    }
    // defect of the time points (u, u_old) with s_m = (1, -1),
    // s_a = (theta dt, (1 - theta) dt) (theta_time_step_impl.h:200-240)
    ug4gb::TimeScale defect_scale() const
    {
        return ug4gb::TimeScale{1.0, theta * dt, -1.0, (1.0 - theta) * dt, u_old.p};
    }
};

// what a multigrid's structure depends on: a re-init with the same key may
// keep the previous level buffers and transfers
struct GmgKey {
    uint64_t g = 0;                       // grid uid
    int nl = 0, base = 0, smoother = 0;
    double damp = 0.0;
    int rap = 0, transposed = 0, precision = 0, allow_dia = 0;
    double damp_prol = 1.0, damp_res = 1.0;
    int smoother2 = 0;
    double damp2 = 0.0;
    int base_kind = 0, base_steps = 0;
    bool operator==(const GmgKey &o) const
    {
        return g && g == o.g && nl == o.nl && base == o.base && smoother == o.smoother && damp == o.damp &&
               rap == o.rap && transposed == o.transposed && precision == o.precision && allow_dia == o.allow_dia &&
               damp_prol == o.damp_prol && damp_res == o.damp_res && smoother2 == o.smoother2 && damp2 == o.damp2 &&
               base_kind == o.base_kind && base_steps == o.base_steps;
    }
};

struct ug4gb_gmg {
    ug4gb_ctx *ctx = nullptr;
    ug4gb_disc *disc = nullptr;
    int smoother = UG4GB_SMOOTHER_JACOBI;   // pre-smoother
    double damp = 0.6;
    int smoother2 = UG4GB_SMOOTHER_JACOBI;  // post-smoother
    double damp2 = 0.6;
    int cycle = 1, nu1 = 2, nu2 = 2, base = 0;
    int base_kind = UG4GB_BASE_LU, base_steps = 10;   // base solver (set_base_solver)
    int precision = UG4GB_PREC_FP64;
    int transposed = 0;
    int rap = 0;                 // coarse operators as Galerkin products R A P (set_rap)
    double damp_prol = 1.0;      // StdTransfer prolongation / restriction damping
    double damp_res = 1.0;
    ug4gb_timedisc *td = nullptr;  // coarse levels assembled as this time discretisation's jacobian
    std::unique_ptr<ug4gb::GmgBase> impl;
    GmgKey built;                // the structure impl was built for
    uint64_t built_settings = 0; // cycle type and smoothing steps impl's graphs were captured with
    int n_top = 0;
    int gen = 0;                 // incremented by every init (invalidates captured graphs)
    // standalone apply graph
    cudaGraphExec_t graph = nullptr;
    const double *graph_d = nullptr;
    double *graph_c = nullptr;
    int64_t graph_kernels = 0;
};

struct ug4gb_solver {
    ug4gb_ctx *ctx = nullptr;
    int kind = UG4GB_SOLVER_CG;
    ug4gb_gmg *pre = nullptr;
    int maxit = 100;
    double min_def = 1e-300, rel_red = 1e-10;
    int num_restarts = 0;        // BiCGStab: restart every num_restarts half steps (0: off)
    double min_ortho = 0.0;      // BiCGStab: restart when (r, r0) <= min_ortho |r| |r0|
    const ug4gb_matrix *A = nullptr;
    uint64_t op_sig = 0;         // device buffers of A's solve format at init
    int n = 0;
    ug4gb::DevBuf<double> r, p, q, r0, v, s, t, zcopy;
    ug4gb::DevBuf<ug4gb::KScal> ks;
    ug4gb::DevBuf<double> hist;
    ug4gb::KScal host_ks{};
    std::vector<double> host_hist;
    // captured solve graph: the prologue, then the iteration loop
    cudaGraphExec_t iter_graph = nullptr;
    int64_t iter_kernels = 0;       // kernels of one loop body
    int64_t prologue_kernels = 0;   // kernels before the loop (entry test included)
    void *pinned = nullptr;         // page-locked read-back of the scalars and the history
    size_t pinned_bytes = 0;
    const double *graph_x = nullptr;
    const double *graph_r = nullptr;
    int graph_pre_gen = -1;
    int last_rc = 0;
};
