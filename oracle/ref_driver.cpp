/*
 * ref_driver.cpp -- runs ugcore's OWN algebra on the oracle's problems.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into
 * oracle/_ref/ref_driver from the reference sources in place (never copied).
 * It pins the C restatement (liboracle) against the reference classes:
 *   ug::SparseMatrix<double> (lib_algebra/cpu_algebra/sparsematrix.h:98):
 *       pattern growth through operator() while adding element matrices in
 *       element order (AddLocalMatrixToGlobal, lib_disc/common/local_algebra.h:767);
 *   ug::SetDirichletRow (lib_algebra/algebra_common/sparsematrix_util.h:850);
 *   ug::SetRow + set_as_transpose_of for P and R
 *       (lagrange_dirichlet_boundary_impl.h:545-752, std_transfer_impl.h:695);
 *   ug::Jacobi, ug::LU (dense), ug::CG, ug::BiCGStab, ug::StdConvCheck.
 * The element matrices and the grid hierarchy come from the restatement
 * (orc_element_matrix / orc_hier_create): the FV1 element discretisation is
 * an external plugin and lib_grid needs Boost, neither is buildable here.
 * The multigrid cycle is the restated AssembledMultiGridCycle control flow
 * (mg_solver_impl.hpp:176-275,1687-2140) driving the reference components.
 *
 * With rap = 1 the coarse level operators are Galerkin products computed by
 * the reference's own ug::AddMultiplyOf(A_c, R, A_f, P)
 * (lib_algebra/algebra_common/sparsematrix_util.h:167), top level down, as
 * AssembledMultiGridCycle::init_rap_operator (mg_solver_impl.hpp:830-1012).
 *
 * Usage: ref_driver <out.bin> elem mx my mz nref seed coef_kind solver vel_kind
 *                   [diffusion peclet smoother damp nu1 nu2 maxit rap]
 * Output (little-endian binary): header ints, per-level CRS, rhs, solution,
 * defect history.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <chrono>

#include "lib_algebra/cpu_algebra_types.h"
#include "lib_algebra/algebra_common/sparsematrix_util.h"
#include "lib_algebra/operator/interface/matrix_operator.h"
#include "lib_algebra/operator/preconditioner/jacobi.h"
#include "lib_algebra/operator/linear_solver/lu.h"
#include "lib_algebra/operator/linear_solver/cg.h"
#include "lib_algebra/operator/linear_solver/bicgstab.h"
#include "lib_algebra/operator/convergence_check.h"

extern "C" {
#include "ug4_oracle.h"
}

using namespace ug;
typedef CPUAlgebra::matrix_type Mat;
typedef CPUAlgebra::vector_type Vec;
typedef MatrixOperator<Mat, Vec> MatOp;

/* Restated multiplicative V/W cycle over reference components. */
class RefGMG : public ILinearIterator<Vec>
{
public:
    int nlev, base, cycle, nu1, nu2;
    double damp_res = 1.0, damp_prol = 1.0;   // StdTransfer::set_restriction/prolongation_damping
    std::vector<SmartPtr<MatOp> > A;
    std::vector<SmartPtr<Mat> > Pp, Rp;
    std::vector<SmartPtr<ILinearIterator<Vec> > > S;
    SmartPtr<ILinearOperatorInverse<Vec> > lu;
    std::vector<Vec> sc, sd, st;

    virtual const char *name() const { return "RefGMG"; }
    virtual bool supports_parallel() const { return false; }
    virtual bool init(SmartPtr<ILinearOperator<Vec> > J, const Vec &u) { return true; }
    virtual bool init(SmartPtr<ILinearOperator<Vec> > L) { return true; }
    virtual SmartPtr<ILinearIterator<Vec> > clone() { return SPNULL; }

    void base_solve(int l)
    {
        lu->apply(sc[l], sd[l]);
        if (l >= nlev - 1) A[l]->apply_sub(sd[l], sc[l]);
    }
    void presmooth_and_restriction(int l)
    {
        for (int nu = 0; nu < nu1; ++nu) {
            S[l]->apply(st[l], sd[l]);
            A[l]->apply_sub(sd[l], st[l]);
            if (nu < nu1 - 1) sc[l] += st[l];
        }
        sc[l - 1].set(0.0);
        if (nu1 > 0) sc[l] += st[l];
        Rp[l]->apply_ignore_zero_rows(sd[l - 1], damp_res, sd[l]);
    }
    void prolongation_and_postsmooth(int l)
    {
        Pp[l]->axpy(st[l], 0.0, st[l], damp_prol, sc[l - 1]);
        sc[l] += st[l];
        for (int nu = 0; nu < nu2; ++nu) {
            A[l]->apply_sub(sd[l], st[l]);
            S[l]->apply(st[l], sd[l]);
            sc[l] += st[l];
        }
        if (l >= nlev - 1) A[l]->apply_sub(sd[l], st[l]);
    }
    void lmgc(int l)
    {
        if (l == base) { base_solve(nlev - 1); return; }
        presmooth_and_restriction(l);
        if (l - 1 == base) base_solve(l - 1);
        else for (int i = 0; i < cycle; ++i) lmgc(l - 1);
        prolongation_and_postsmooth(l);
    }
    virtual bool apply(Vec &c, const Vec &d)
    {
        int top = nlev - 1;
        for (size_t i = 0; i < d.size(); ++i) sd[top][i] = d[i];
        c.set(0.0);
        sc[top].set(0.0);
        lmgc(top);
        for (size_t i = 0; i < c.size(); ++i) c[i] += sc[top][i];
        return true;
    }
    virtual bool apply_update_defect(Vec &c, Vec &d)
    {
        apply(c, d);
        A[nlev - 1]->apply_sub(d, c);
        return true;
    }
};

/* StdConvCheck that records the defect history without printing */
class RecConv : public StdConvCheck<Vec>
{
public:
    std::vector<double> h;
    RecConv(int maxit, number mind, number red) : StdConvCheck<Vec>(maxit, mind, red, false) {}
    virtual void start_defect(number d) { StdConvCheck<Vec>::start_defect(d); h.clear(); h.push_back(d); }
    virtual void update_defect(number d) { StdConvCheck<Vec>::update_defect(d); h.push_back(d); }
};

static void write_crs(FILE *f, const Mat &M)
{
    int n = (int)M.num_rows();
    std::vector<int> rp(n + 1, 0), ci;
    std::vector<double> va;
    for (int r = 0; r < n; ++r) {
        for (Mat::const_row_iterator it = M.begin_row(r); it != M.end_row(r); ++it) {
            ci.push_back((int)it.index());
            va.push_back(it.value());
        }
        rp[r + 1] = (int)ci.size();
    }
    int64_t nnz = (int64_t)ci.size();
    fwrite(&n, sizeof(int), 1, f);
    fwrite(&nnz, sizeof(int64_t), 1, f);
    fwrite(rp.data(), sizeof(int), n + 1, f);
    fwrite(ci.data(), sizeof(int), ci.size(), f);
    fwrite(va.data(), sizeof(double), va.size(), f);
}

int main(int argc, char **argv)
{
    if (argc < 11) {
        fprintf(stderr, "usage: ref_driver out.bin elem mx my mz nref seed coef_kind solver vel_kind "
                        "[diffusion peclet smoother damp nu1 nu2 maxit rap bicg_restart bicg_min_ortho damp_prol damp_res]\n");
        return 2;
    }
    const char *out = argv[1];
    int elem = atoi(argv[2]), mx = atoi(argv[3]), my = atoi(argv[4]), mz = atoi(argv[5]);
    int nref = atoi(argv[6]);
    uint64_t seed = strtoull(argv[7], 0, 10);
    int coef_kind = atoi(argv[8]), solver = atoi(argv[9]), vel_kind = atoi(argv[10]);
    double diffusion = argc > 11 ? atof(argv[11]) : 1.0;
    double peclet = argc > 12 ? atof(argv[12]) : 10.0;
    double damp = argc > 14 ? atof(argv[14]) : 0.6;
    int nu1 = argc > 15 ? atoi(argv[15]) : 2, nu2 = argc > 16 ? atoi(argv[16]) : 2;
    int maxit = argc > 17 ? atoi(argv[17]) : 200;
    int rap = argc > 18 ? atoi(argv[18]) : 0;
    int bicg_restart = argc > 19 ? atoi(argv[19]) : 0;
    double bicg_min_ortho = argc > 20 ? atof(argv[20]) : 0.0;
    double damp_prol = argc > 21 ? atof(argv[21]) : 1.0, damp_res = argc > 22 ? atof(argv[22]) : 1.0;

    orc_hier H;
    if (orc_hier_create(&H, elem, mx, my, mz, nref)) return 3;
    int nl = H.nlev, top = nl - 1;
    std::vector<double *> K(nl);
    if (coef_kind == 3) {
        for (int l = 0; l < nl; ++l) {
            K[l] = (double *)malloc(sizeof(double) * H.lev[l].ne);
            for (int e = 0; e < H.lev[l].ne; ++e) K[l][e] = diffusion;
        }
    } else {
        orc_problem pr;
        memset(&pr, 0, sizeof(pr));
        pr.seed = seed; pr.coef_kind = coef_kind; pr.coef_modes = 64; pr.coef_kmax = 8.0;
        orc_problem_coefficients(&pr, &H, K.data());
    }
    orc_field vf;
    int upwind = 0;
    if (vel_kind == 1) {
        orc_field_curl_init(&vf, 16, 2.0, seed ^ 0x7E10C17ULL);
        vf.scale *= peclet * 2.0 * diffusion * (double)(H.lev[top].nx - 1);
        upwind = 1;
    }
    std::vector<double> f(H.lev[top].nv);
    orc_source_uniform(seed, H.lev[top].nv, f.data());

    auto t0 = std::chrono::steady_clock::now();
    RefGMG *G = new RefGMG;
    SmartPtr<ILinearIterator<Vec> > spG(G);
    G->nlev = nl; G->base = 0; G->cycle = 1; G->nu1 = nu1; G->nu2 = nu2;
    G->damp_prol = damp_prol; G->damp_res = damp_res;
    G->A.resize(nl); G->Pp.resize(nl); G->Rp.resize(nl); G->S.resize(nl);
    G->sc.resize(nl); G->sd.resize(nl); G->st.resize(nl);
    Vec b;
    double Aloc[64], vol[8];
    for (int l = 0; l < nl; ++l) {
        const orc_level &L = H.lev[l];
        G->A[l] = make_sp(new MatOp);
        Mat &M = G->A[l]->get_matrix();
        M.resize_and_clear(L.nv, L.nv);
        if (l == top) { b.resize(L.nv); b.set(0.0); }
        for (int e = 0; e < L.ne; ++e) {
            orc_element_matrix(&L, e, K[l][e], upwind ? &vf : NULL, upwind, Aloc, vol);
            const int *ev = L.elems + (size_t)e * L.k;
            for (int i = 0; i < L.k; ++i)
                for (int j = 0; j < L.k; ++j) M(ev[i], ev[j]) += Aloc[i * L.k + j];
            if (l == top)
                for (int i = 0; i < L.k; ++i) b[ev[i]] += f[ev[i]] * vol[i];
        }
        for (int v = 0; v < L.nv; ++v)
            if (L.bnd[v]) { SetDirichletRow(M, v); if (l == top) b[v] = 0.0; }
        M.defragment();
        G->sc[l].resize(L.nv); G->sd[l].resize(L.nv); G->st[l].resize(L.nv);
        G->sc[l].set(0.0); G->sd[l].set(0.0); G->st[l].set(0.0);
        if (l > 0) {
            G->Pp[l] = make_sp(new Mat); Mat &Pm = *G->Pp[l];
            Pm.resize_and_clear(L.nv, H.lev[l - 1].nv);
            for (int v = 0; v < L.nv; ++v) {
                int n = L.npar[v];
                double w = (n == 1) ? 1.0 : (n == 2 ? 0.5 : (n == 4 ? 0.25 : 0.125));
                for (int j = 0; j < n; ++j) Pm(v, L.par[8 * (size_t)v + j]) = w;
            }
            for (int v = 0; v < L.nv; ++v) {
                if (!L.bnd[v]) continue;
                SetRow(Pm, v, 0.0);
                if (L.npar[v] == 1) Pm(v, L.par[8 * (size_t)v]) = 1.0;
            }
            G->Rp[l] = make_sp(new Mat); Mat &Rm = *G->Rp[l];
            Rm.set_as_transpose_of(Pm);
            for (int v = 0; v < L.nv; ++v) {
                if (!L.bnd[v] || L.npar[v] != 1) continue;
                int c = L.par[8 * (size_t)v];
                SetRow(Rm, c, 0.0);
                Rm(c, v) = 1.0;
            }
            Pm.defragment(); Rm.defragment();
        }
    }
    if (rap) {
        for (int l = top; l > 0; --l) {
            Mat &Ac = G->A[l - 1]->get_matrix();
            Ac.resize_and_clear(H.lev[l - 1].nv, H.lev[l - 1].nv);
            AddMultiplyOf(Ac, *G->Rp[l], G->A[l]->get_matrix(), *G->Pp[l]);
            Ac.defragment();
        }
    }
    for (int l = 1; l < nl; ++l) {
        G->S[l] = SmartPtr<ILinearIterator<Vec> >(new Jacobi<CPUAlgebra>(damp));
        G->S[l]->init(G->A[l]);
    }
    G->lu = SmartPtr<ILinearOperatorInverse<Vec> >(new LU<CPUAlgebra>);
    G->lu->init(G->A[0]);
    auto t1 = std::chrono::steady_clock::now();

    SmartPtr<RecConv> conv = make_sp(new RecConv(maxit, 1e-300, 1e-10));
    Vec x(H.lev[top].nv);
    x.set(0.0);
    Vec rhs(b.size());
    for (size_t i = 0; i < b.size(); ++i) rhs[i] = b[i];
    std::vector<double> hist;
    bool ok;
    if (solver == 0) {
        CG<Vec> cg;
        cg.set_preconditioner(spG);
        cg.set_convergence_check(conv);
        cg.init(G->A[top]);
        ok = cg.apply_return_defect(x, rhs);
    } else {
        BiCGStab<Vec> bi;
        bi.set_restart(bicg_restart);
        bi.set_min_orthogonality(bicg_min_ortho);
        bi.set_preconditioner(spG);
        bi.set_convergence_check(conv);
        bi.init(G->A[top]);
        ok = bi.apply_return_defect(x, rhs);
    }
    auto t2 = std::chrono::steady_clock::now();
    hist = conv->h;
    int steps = conv->step();
    double d0 = hist.empty() ? 0.0 : hist[0], d1 = conv->defect();

    FILE *fo = fopen(out, "wb");
    if (!fo) return 4;
    int hdr[4] = {nl, steps, ok ? 1 : 0, (int)hist.size()};
    fwrite(hdr, sizeof(int), 4, fo);
    double dd[4] = {d0, d1, std::chrono::duration<double>(t1 - t0).count(),
                    std::chrono::duration<double>(t2 - t1).count()};
    fwrite(dd, sizeof(double), 4, fo);
    for (int l = 0; l < nl; ++l) write_crs(fo, G->A[l]->get_matrix());
    for (int l = 1; l < nl; ++l) { write_crs(fo, *G->Pp[l]); write_crs(fo, *G->Rp[l]); }
    fwrite(&b[0], sizeof(double), b.size(), fo);
    fwrite(&x[0], sizeof(double), x.size(), fo);
    if (!hist.empty()) fwrite(hist.data(), sizeof(double), hist.size(), fo);
    fclose(fo);
    printf("steps %d ok %d d0 %.6e d1 %.6e setup %.3fs solve %.3fs\n", steps, ok ? 1 : 0, d0, d1,
           dd[2], dd[3]);
    return 0;
}
