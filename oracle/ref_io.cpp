/*
 * ref_io.cpp -- runs ugcore's OWN matrix/vector file writers and readers.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh into
 * oracle/_ref/ref_io from the reference sources in place (never copied):
 *   ug::MatrixIOMtx (lib_algebra/common/matrixio/matrix_io_mtx.h:59,
 *       matrix_io_mtx.cpp) -- write_from as SaveMatrixToMTX does
 *       (lib_disc/function_spaces/grid_function_util.h:761-778), read_into;
 *   ug::ConnectionViewer::WriteMatrix / WriteVector
 *       (lib_algebra/common/connection_viewer_output.h:114-140,395-420),
 *       ReadVector (lib_algebra/common/connection_viewer_input.h:104-150).
 * The files it writes are committed as fixtures (tests/golden/io/) by
 * tests/golden/make_io_golden.py; the library's own writers must reproduce
 * them byte for byte and its readers must return what ugcore's read.
 *
 * Binary inputs/outputs (little endian):
 *   CRS:       int32 rows, int32 cols, int64 nnz, int32 rowptr[rows+1],
 *              int32 col[nnz], float64 val[nnz]
 *   positions: int32 n, int32 dim, float64 xyz[n*dim]
 *   vector:    int32 n, float64 v[n]
 *
 * Usage:
 *   ref_io write-mtx  A.csr out.mtx [comment]    (no comment argument: the default)
 *   ref_io read-mtx   in.mtx out.csr
 *   ref_io write-mat  A.csr pos.bin out.mat
 *   ref_io write-vec  v.bin pos.bin out.vec
 *   ref_io write-vec-diff  v.bin w.bin pos.bin out.vec   (WriteVector with compareVec: v - w)
 *   ref_io read-vec   in.vec n out.bin
 */
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lib_algebra/cpu_algebra_types.h"
#include "lib_algebra/common/matrixio/matrix_io_mtx.h"
#include "lib_algebra/common/connection_viewer_output.h"
#include "lib_algebra/common/connection_viewer_input.h"
#include "common/math/ugmath_types.h"

using namespace ug;
typedef CPUAlgebra::matrix_type Mat;
typedef CPUAlgebra::vector_type Vec;

static bool read_file(const char *path, std::vector<char> &buf)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    buf.resize((size_t)n);
    bool ok = fread(buf.data(), 1, (size_t)n, f) == (size_t)n;
    fclose(f);
    return ok;
}

static bool load_crs(const char *path, Mat &A)
{
    std::vector<char> b;
    if (!read_file(path, b) || b.size() < 16) return false;
    int32_t rows, cols;
    int64_t nnz;
    memcpy(&rows, &b[0], 4);
    memcpy(&cols, &b[4], 4);
    memcpy(&nnz, &b[8], 8);
    const int32_t *rp = (const int32_t *)&b[16];
    const int32_t *ci = rp + rows + 1;
    const double *va = (const double *)(ci + nnz);
    A.resize_and_clear(rows, cols);
    for (int r = 0; r < rows; ++r)
        for (int a = rp[r]; a < rp[r + 1]; ++a) A(r, ci[a]) = va[a];
    A.defragment();
    return true;
}

static bool save_crs(const char *path, const Mat &A)
{
    FILE *f = fopen(path, "wb");
    if (!f) return false;
    int32_t rows = (int32_t)A.num_rows(), cols = (int32_t)A.num_cols();
    std::vector<int32_t> rp(rows + 1, 0), ci;
    std::vector<double> va;
    for (int r = 0; r < rows; ++r) {
        for (Mat::const_row_iterator it = A.begin_row(r); it != A.end_row(r); ++it) {
            ci.push_back((int32_t)it.index());
            va.push_back(it.value());
        }
        rp[r + 1] = (int32_t)ci.size();
    }
    int64_t nnz = (int64_t)ci.size();
    fwrite(&rows, 4, 1, f);
    fwrite(&cols, 4, 1, f);
    fwrite(&nnz, 8, 1, f);
    fwrite(rp.data(), 4, rp.size(), f);
    fwrite(ci.data(), 4, ci.size(), f);
    fwrite(va.data(), 8, va.size(), f);
    fclose(f);
    return true;
}

template <int dim>
static bool load_positions(const std::vector<char> &b, std::vector<MathVector<dim> > &pos)
{
    int32_t n, d;
    memcpy(&n, &b[0], 4);
    memcpy(&d, &b[4], 4);
    if (d != dim) return false;
    const double *x = (const double *)&b[8];
    pos.resize(n);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < dim; ++k) pos[i][k] = x[(size_t)i * dim + k];
    return true;
}

static int pos_dim(const std::vector<char> &b)
{
    int32_t d;
    memcpy(&d, &b[4], 4);
    return d;
}

template <int dim>
static int write_mat(const Mat &A, const std::vector<char> &pb, const char *out)
{
    std::vector<MathVector<dim> > pos;
    if (!load_positions<dim>(pb, pos)) return 3;
    ConnectionViewer::WriteMatrix(std::string(out), A, &pos[0], dim);
    return 0;
}

template <int dim>
static int write_vec(const Vec &v, const std::vector<char> &pb, const char *out, const Vec *cmp = NULL)
{
    std::vector<MathVector<dim> > pos;
    if (!load_positions<dim>(pb, pos)) return 3;
    ConnectionViewer::WriteVector(std::string(out), v, &pos[0], dim, cmp);
    return 0;
}

static bool load_vec(const char *path, Vec &v)
{
    std::vector<char> vb;
    if (!read_file(path, vb)) return false;
    int32_t n;
    memcpy(&n, &vb[0], 4);
    v.resize(n);
    const double *x = (const double *)&vb[4];
    for (int i = 0; i < n; ++i) v[i] = x[i];
    return true;
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: see the header of ref_io.cpp\n");
        return 2;
    }
    const std::string cmd = argv[1];
    try {
        if (cmd == "write-mtx") {
            Mat A;
            if (!load_crs(argv[2], A)) return 3;
            // SaveMatrixToMTX: EXISTING when the file is there, else NEW
            FILE *probe = fopen(argv[3], "r");
            const int mode = probe ? MatrixIO::EXISTING : MatrixIO::NEW;
            if (probe) fclose(probe);
            MatrixIOMtx mtx(argv[3], mode);
            if (argc > 4) mtx.write_from(A, std::string(argv[4]));
            else mtx.write_from(A);
            return 0;
        }
        if (cmd == "read-mtx") {
            MatrixIOMtx mtx(argv[2], MatrixIO::EXISTING);
            Mat A;
            mtx.read_into(A);
            A.defragment();
            return save_crs(argv[3], A) ? 0 : 3;
        }
        if (cmd == "write-mat" && argc >= 5) {
            Mat A;
            std::vector<char> pb;
            if (!load_crs(argv[2], A) || !read_file(argv[3], pb)) return 3;
            switch (pos_dim(pb)) {
                case 1: return write_mat<1>(A, pb, argv[4]);
                case 2: return write_mat<2>(A, pb, argv[4]);
                case 3: return write_mat<3>(A, pb, argv[4]);
            }
            return 3;
        }
        if (cmd == "write-vec" && argc >= 5) {
            std::vector<char> vb, pb;
            if (!read_file(argv[2], vb) || !read_file(argv[3], pb)) return 3;
            int32_t n;
            memcpy(&n, &vb[0], 4);
            Vec v(n);
            const double *x = (const double *)&vb[4];
            for (int i = 0; i < n; ++i) v[i] = x[i];
            switch (pos_dim(pb)) {
                case 1: return write_vec<1>(v, pb, argv[4]);
                case 2: return write_vec<2>(v, pb, argv[4]);
                case 3: return write_vec<3>(v, pb, argv[4]);
            }
            return 3;
        }
        if (cmd == "write-vec-diff" && argc >= 6) {
            Vec v, w;
            std::vector<char> pb;
            if (!load_vec(argv[2], v) || !load_vec(argv[3], w) || !read_file(argv[4], pb)) return 3;
            switch (pos_dim(pb)) {
                case 1: return write_vec<1>(v, pb, argv[5], &w);
                case 2: return write_vec<2>(v, pb, argv[5], &w);
                case 3: return write_vec<3>(v, pb, argv[5], &w);
            }
            return 3;
        }
        if (cmd == "read-vec" && argc >= 5) {
            const int n = atoi(argv[3]);
            Vec v(n);
            for (int i = 0; i < n; ++i) v[i] = 0.0;
            if (!ConnectionViewer::ReadVector(std::string(argv[2]), v)) return 4;
            FILE *f = fopen(argv[4], "wb");
            if (!f) return 3;
            int32_t m = (int32_t)v.size();
            fwrite(&m, 4, 1, f);
            for (int i = 0; i < m; ++i) fwrite(&v[i], 8, 1, f);
            fclose(f);
            return 0;
        }
    } catch (const std::exception &e) {
        fprintf(stderr, "ref_io: %s\n", e.what());
        return 5;
    } catch (...) {
        fprintf(stderr, "ref_io: ugcore error\n");
        return 5;
    }
    fprintf(stderr, "ref_io: unknown command %s\n", cmd.c_str());
    return 2;
}
