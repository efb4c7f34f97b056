/*
 * ref_smoothers.cpp -- runs ugcore's OWN ILU(0) and Gauss-Seidel smoothers
 * with a given row ordering on a matrix read from a file.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into
 * oracle/_ref/ref_smoothers from the reference sources in place (never
 * copied).  It pins the oracle's multicolour smoothers (oracle/
 * ug4_oracle_solve.c: ilu_factor / ilu_apply, mcgs_apply, mcgs_backward,
 * mcsgs_backward, all sweeping rows in (colour, index) order) against:
 *   ug::ILU<CPUAlgebra> (lib_algebra/operator/preconditioner/ilu.h:321-735)
 *       given the ordering through ILU::set_ordering_algorithm (:396):
 *       ILU::apply_ordering (:430-462) permutes the matrix with
 *       SetMatrixAsPermutation (lib_algebra/algebra_common/
 *       permutation_util.h:50), FactorizeILUSorted (ilu.h:174) factorises it
 *       in index order, and step (:580-615) permutes the defect, runs
 *       invert_L / invert_U (:233-318) and permutes the correction back;
 *   ug::GaussSeidel, ug::SymmetricGaussSeidel, ug::BackwardGaussSeidel
 *       (gauss_seidel.h:271,350,316; gs_step_LL / sgs_step / gs_step_UR,
 *       lib_algebra/algebra_common/core_smoothers.h:106-206) with
 *       set_sor_relax (:96).  Their serial step sweeps in index order and does
 *       not use an ordering algorithm, so they are run on the permuted system
 *       (SetMatrixAsPermutation, SetVectorAsPermutation) and the correction
 *       is permuted back here;
 *   ug::Jacobi (jacobi.h:90) with its damping, in any order;
 *   and, with steps = k > 0, each of them as the base solver a script sets
 *       with gmg:set_base_solver: ug::LinearSolver (linear_solver/
 *       linear_solver.h:114-190) with StdConvCheck(k, 0, 0, false, true)
 *       (convergence_check.h:185): k corrections c = B d, x += c, d -= A c.
 *
 * Usage: ref_smoothers <in.bin> <out.bin>
 * in.bin (little-endian): int32 n, int64 nnz, int32 rowptr[n+1],
 *   int32 col[nnz], float64 val[nnz], int64 perm[n] (old index i -> new
 *   index perm[i]), int32 kind (0 ILU, 1 GaussSeidel, 2 SymmetricGaussSeidel,
 *   3 BackwardGaussSeidel, 4 Jacobi), float64 relax (SOR factor / Jacobi
 *   damping), int32 steps (0: one application), int32 nvec, float64 d[nvec][n].
 * out.bin: float64 c[nvec][n], c = B d of that smoother (steps = 0) or the
 *   LinearSolver's x after k steps from x = 0.
 */
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "lib_algebra/cpu_algebra_types.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/preconditioner/ilu.h"
#include "lib_algebra/operator/preconditioner/gauss_seidel.h"
#include "lib_algebra/algebra_common/permutation_util.h"
#include "lib_algebra/operator/preconditioner/jacobi.h"
#include "lib_algebra/operator/linear_solver/linear_solver.h"
#include "lib_algebra/operator/convergence_check.h"

using namespace ug;
typedef CPUAlgebra::matrix_type Mat;
typedef CPUAlgebra::vector_type Vec;
typedef MatrixOperator<Mat, Vec> MatOp;
typedef std::vector<size_t> Ordering;

/* an ordering algorithm that hands ILU a fixed permutation */
class FixedOrdering : public IOrderingAlgorithm<CPUAlgebra, Ordering>
{
    Ordering o;

public:
    explicit FixedOrdering(const Ordering &p) : o(p) {}
    void compute() override {}
    void check() override {}
    Ordering &ordering() override { return o; }
    void init(M_t *) override {}
    void init(M_t *, const V_t &) override {}
    void init(M_t *, const std::vector<size_t> &) override {}
    void init(M_t *, const V_t &, const std::vector<size_t> &) override {}
    SmartPtr<IOrderingAlgorithm<CPUAlgebra, Ordering> > clone() override { return make_sp(new FixedOrdering(o)); }
    const char *name() const override { return "fixed"; }
};

template <class T>
static void rd(FILE *f, T *p, size_t n)
{
    if (fread(p, sizeof(T), n, f) != n) {
        fprintf(stderr, "ref_smoothers: short input\n");
        exit(2);
    }
}

int main(int argc, char **argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: ref_smoothers in.bin out.bin\n");
        return 2;
    }
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t n;
    int64_t nnz;
    rd(f, &n, 1);
    rd(f, &nnz, 1);
    std::vector<int32_t> rp(n + 1), ci(nnz);
    std::vector<double> va(nnz);
    std::vector<int64_t> perm(n);
    rd(f, rp.data(), rp.size());
    rd(f, ci.data(), ci.size());
    rd(f, va.data(), va.size());
    rd(f, perm.data(), perm.size());
    int32_t kind, steps;
    double relax;
    rd(f, &kind, 1);
    rd(f, &relax, 1);
    rd(f, &steps, 1);
    int32_t nvec;
    rd(f, &nvec, 1);
    std::vector<double> d((size_t)nvec * n);
    rd(f, d.data(), d.size());
    fclose(f);

    SmartPtr<MatOp> op = make_sp(new MatOp);
    Mat &A = op->get_matrix();
    A.resize_and_clear(n, n);
    for (int r = 0; r < n; ++r)
        for (int a = rp[r]; a < rp[r + 1]; ++a) A(r, ci[a]) = va[a];
    A.defragment();
    const Ordering ord(perm.begin(), perm.end());

    SmartPtr<ILinearIterator<Vec> > sm;
    SmartPtr<MatOp> run_op = op;
    if (kind == 0) {
        SmartPtr<ILU<CPUAlgebra> > ilu = make_sp(new ILU<CPUAlgebra>());
        ilu->set_ordering_algorithm(make_sp(new FixedOrdering(ord)));
        sm = ilu;
    } else {
        /* the permuted system PA = P A P^T */
        run_op = make_sp(new MatOp);
        SetMatrixAsPermutation(run_op->get_matrix(), A, ord);
        run_op->get_matrix().defragment();
        if (kind == 1) {
            SmartPtr<GaussSeidel<CPUAlgebra> > gs = make_sp(new GaussSeidel<CPUAlgebra>());
            gs->set_sor_relax(relax);
            sm = gs;
        } else if (kind == 2) {
            SmartPtr<SymmetricGaussSeidel<CPUAlgebra> > gs = make_sp(new SymmetricGaussSeidel<CPUAlgebra>());
            gs->set_sor_relax(relax);
            sm = gs;
        } else if (kind == 4) {
            sm = make_sp(new Jacobi<CPUAlgebra>(relax));
        } else {
            SmartPtr<BackwardGaussSeidel<CPUAlgebra> > gs = make_sp(new BackwardGaussSeidel<CPUAlgebra>());
            gs->set_sor_relax(relax);
            sm = gs;
        }
    }
    if (steps > 0) {
        /* the smoother as the base solver: k steps of a LinearSolver */
        SmartPtr<LinearSolver<Vec> > ls = make_sp(new LinearSolver<Vec>());
        ls->set_preconditioner(sm);
        ls->set_convergence_check(make_sp(new StdConvCheck<Vec>(steps, 0.0, 0.0, false, true)));
        if (!ls->init(run_op)) {
            fprintf(stderr, "ref_smoothers: LinearSolver::init failed\n");
            return 1;
        }
        FILE *g = fopen(argv[2], "wb");
        if (!g) return 2;
        Vec dv(n), cv(n), pd(n), pc(n);
        for (int v = 0; v < nvec; ++v) {
            for (int i = 0; i < n; ++i) dv[i] = d[(size_t)v * n + i];
            if (kind == 0) {
                cv.set(0.0);
                if (!ls->apply(cv, dv)) return 1;
            } else {
                SetVectorAsPermutation(pd, dv, ord);
                pc.set(0.0);
                if (!ls->apply(pc, pd)) return 1;
                for (int i = 0; i < n; ++i) cv[i] = pc[ord[i]];
            }
            for (int i = 0; i < n; ++i) fwrite(&cv[i], sizeof(double), 1, g);
        }
        fclose(g);
        return 0;
    }
    /* through the public interface a linear solver uses */
    SmartPtr<ILinearOperator<Vec> > lop = run_op;
    if (!sm->init(lop)) {
        fprintf(stderr, "ref_smoothers: init failed\n");
        return 1;
    }
    FILE *g = fopen(argv[2], "wb");
    if (!g) return 2;
    Vec dv(n), cv(n), pd(n), pc(n);
    for (int v = 0; v < nvec; ++v) {
        for (int i = 0; i < n; ++i) dv[i] = d[(size_t)v * n + i];
        cv.set(0.0);
        if (kind == 0) {
            if (!sm->apply(cv, dv)) {
                fprintf(stderr, "ref_smoothers: apply failed\n");
                return 1;
            }
        } else {
            SetVectorAsPermutation(pd, dv, ord);
            pc.set(0.0);
            if (!sm->apply(pc, pd)) {
                fprintf(stderr, "ref_smoothers: apply failed\n");
                return 1;
            }
            for (int i = 0; i < n; ++i) cv[i] = pc[ord[i]];
        }
        for (int i = 0; i < n; ++i) fwrite(&cv[i], sizeof(double), 1, g);
    }
    fclose(g);
    return 0;
}
