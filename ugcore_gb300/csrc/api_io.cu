// api_io.cu -- matrix and vector files in the two formats ugcore writes:
//
//   MatrixMarket coordinate files (SaveMatrixToMTX,
//   lib_disc/function_spaces/grid_function_util.h:761-778, over MatrixIOMtx,
//   lib_algebra/common/matrixio/matrix_io_mtx.h:243-371 and
//   matrix_io_mtx.cpp:170-303): the writer detects symmetry and
//   skew-symmetry exactly, writes only the lower triangle of such matrices,
//   skips zero values and lists the entries column by column; the reader
//   mirrors symmetric / skew-symmetric entries and lets a later assignment to
//   the same position replace an earlier one.
//
//   ConnectionViewer files (.mat / .vec: ConnectionViewer::WriteMatrix and
//   WriteVector, lib_algebra/common/connection_viewer_output.h:95-140,395-420;
//   ReadVector, connection_viewer_input.h:104-150): a grid header with one
//   position per row, then one "row col value" line per stored entry.
//
// Files are byte-identical to ugcore's: every number is printed with the
// printf conversion that the C++ stream settings of the reference select
// ("%.13e" for MatrixMarket values, "%g" for ConnectionViewer matrices and
// positions, "%.16g" for ConnectionViewer vectors).
//
// This is host code.  The matrix / vector entry points copy the device CRS
// or vector to the host (or back) and call the host-array entry points, which
// need no CUDA context and format the text on all host threads.
#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "gmg.cuh"

namespace {

struct IoError {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw IoError{code, buf};
}

template <class F>
int io_guarded(char *err, int cap, F &&f)
{
    try {
        f();
        return UG4GB_OK;
    } catch (const IoError &e) {
        if (err && cap > 0) snprintf(err, (size_t)cap, "%s", e.msg.c_str());
        return e.code;
    } catch (const ug4gb::Error &e) {
        if (err && cap > 0) snprintf(err, (size_t)cap, "%s", e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc &) {
        if (err && cap > 0) snprintf(err, (size_t)cap, "out of host memory");
        return UG4GB_ERR_NOMEM;
    }
}

// FileTypeIs (common/util/file_util.cpp:86-91): the text from the last '.' on
bool file_type_is(const char *name, const char *ext)
{
    const char *dot = strrchr(name, '.');
    return dot && strcmp(dot, ext) == 0;
}

int num_threads()
{
    const unsigned h = std::thread::hardware_concurrency();
    return (int)std::max(1u, std::min(h, 64u));
}

// Runs body(t, lo, hi) over [0, n) in contiguous chunks on up to num_threads()
// threads (one chunk per thread; small n stays on the calling thread).
template <class F>
void parallel_chunks(int64_t n, int64_t min_per_thread, F &&body)
{
    int T = (int)std::min<int64_t>(num_threads(), std::max<int64_t>(1, n / std::max<int64_t>(1, min_per_thread)));
    if (T <= 1) {
        body(0, (int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t) {
        const int64_t lo = n * t / T, hi = n * (t + 1) / T;
        th.emplace_back([&, t, lo, hi] { body(t, lo, hi); });
    }
    for (auto &x : th) x.join();
}

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) : f(fopen(path, mode)) {}
    ~File()
    {
        if (f) fclose(f);
    }
    void write(const std::string &s, const char *path)
    {
        if (!s.empty() && fwrite(s.data(), 1, s.size(), f) != s.size()) fail(UG4GB_ERR_INVALID, "%s: write failed", path);
    }
};

void check_csr(int rows, int cols, const int *rp, const int *ci)
{
    if (rows < 0 || cols < 0 || !rp) fail(UG4GB_ERR_INVALID, "CRS: bad sizes");
    if (rp[0] != 0) fail(UG4GB_ERR_INVALID, "CRS: rowptr[0] != 0");
    for (int r = 0; r < rows; ++r) {
        if (rp[r + 1] < rp[r]) fail(UG4GB_ERR_INVALID, "CRS: row pointers decrease at row %d", r);
        for (int a = rp[r]; a < rp[r + 1]; ++a) {
            if (ci[a] < 0 || ci[a] >= cols) fail(UG4GB_ERR_INVALID, "CRS: column %d out of range in row %d", ci[a], r);
            if (a > rp[r] && ci[a] <= ci[a - 1])
                fail(UG4GB_ERR_INVALID, "CRS: columns of row %d are not strictly increasing", r);
        }
    }
}

// A(r, c) of a CRS with sorted rows, 0 where nothing is stored (SparseMatrix's
// const operator(), sparsematrix.h:265-290).  Rows past the end read as empty.
inline double crs_at(int rows, const int *rp, const int *ci, const double *va, int r, int c)
{
    if (r < 0 || r >= rows) return 0.0;
    const int *b = ci + rp[r], *e = ci + rp[r + 1];
    const int *p = std::lower_bound(b, e, c);
    return (p != e && *p == c) ? va[p - ci] : 0.0;
}

// ------------------------------------------------------------ MatrixMarket --
enum MtxSym { MTX_GENERAL = 0, MTX_SYMMETRIC = 1, MTX_SKEW = 2 };

void mtx_write(int rows, int cols, const int *rp, const int *ci, const double *va, const char *path,
               const char *comment_in)
{
    if (!path || !file_type_is(path, ".mtx"))
        fail(UG4GB_ERR_INVALID,
             "Please use '.mtx' as file extension for MatrixMarket exchange files. (Filename is '%s')",
             path ? path : "(null)");
    check_csr(rows, cols, rp, ci);
    // determine_matrix_characteristics (matrix_io_mtx.h:297-371): symmetric /
    // skew-symmetric over the nonzero off-diagonal entries, exact comparisons
    const int T = num_threads();
    std::vector<char> sym_t(T, 1), skew_t(T, 1);
    std::vector<int64_t> diag_t(T, 0), off_t(T, 0);
    parallel_chunks(rows, 4096, [&](int t, int64_t lo, int64_t hi) {
        bool sym = true, skew = true;
        int64_t nd = 0, no = 0;
        for (int64_t r = lo; r < hi; ++r)
            for (int a = rp[r]; a < rp[r + 1]; ++a) {
                const double v = va[a];
                if (!(v != 0.0)) continue;
                if (ci[a] == r) {
                    ++nd;
                    continue;
                }
                ++no;
                const double w = crs_at(rows, rp, ci, va, ci[a], (int)r);
                if (v != w) sym = false;
                if (v != -1.0 * w) skew = false;
            }
        sym_t[t] = sym;
        skew_t[t] = skew;
        diag_t[t] = nd;
        off_t[t] = no;
    });
    bool sym = true, skew = true;
    int64_t nd = 0, no = 0;
    for (int t = 0; t < T; ++t) {
        sym = sym && sym_t[t];
        skew = skew && skew_t[t];
        nd += diag_t[t];
        no += off_t[t];
    }
    // a matrix that is both (no nonzero off-diagonal entry) is written as symmetric
    const int kind = sym ? MTX_SYMMETRIC : (skew ? MTX_SKEW : MTX_GENERAL);
    const bool lower = kind != MTX_GENERAL;
    const int64_t lines = lower ? no / 2 + nd : no + nd;

    // entries column by column, rows ascending within a column
    std::vector<int64_t> cstart((size_t)cols + 1, 0);
    for (int r = 0; r < rows; ++r)
        for (int a = rp[r]; a < rp[r + 1]; ++a)
            if (va[a] != 0.0 && (!lower || ci[a] <= r)) ++cstart[(size_t)ci[a] + 1];
    for (int c = 0; c < cols; ++c) cstart[c + 1] += cstart[c];
    const int64_t m = cstart[cols];
    std::vector<int> er((size_t)m);
    std::vector<double> ev((size_t)m);
    {
        std::vector<int64_t> pos(cstart.begin(), cstart.end() - 1);
        for (int r = 0; r < rows; ++r)
            for (int a = rp[r]; a < rp[r + 1]; ++a)
                if (va[a] != 0.0 && (!lower || ci[a] <= r)) {
                    const int64_t p = pos[ci[a]]++;
                    er[p] = r;
                    ev[p] = va[a];
                }
    }
    std::vector<int> ecol((size_t)m);
    for (int c = 0; c < cols; ++c)
        for (int64_t p = cstart[c]; p < cstart[c + 1]; ++p) ecol[p] = c;

    // header: banner (write_banner, matrix_io_mtx.cpp:270-285), comment, sizes
    std::string head = "%%MatrixMarket matrix coordinate real ";
    head += kind == MTX_GENERAL ? "general" : (kind == MTX_SYMMETRIC ? "symmetric" : "skew-symmetric");
    head += "\n";
    std::string comment = comment_in ? comment_in : "%Generated with ug4.";
    if (!comment.empty()) {
        if (comment.find_first_of('%') != 0) comment.insert(0, "%");
        head += comment + "\n";
    }
    char line[96];
    snprintf(line, sizeof line, "%d %d %lld\n", rows, cols, (long long)lines);
    head += line;

    // data lines (write_entry, matrix_io_mtx.cpp:287-300): "row col" 1-based,
    // one extra blank before a non-negative value, %.13e
    std::vector<std::string> parts(T);
    parallel_chunks(m, 1 << 14, [&](int t, int64_t lo, int64_t hi) {
        std::string &s = parts[t];
        s.reserve((size_t)(hi - lo) * 32);
        char b[96];
        for (int64_t p = lo; p < hi; ++p) {
            const double v = ev[p];
            const int n = snprintf(b, sizeof b, "%d %d%s%.13e\n", er[p] + 1, ecol[p] + 1, v < 0 ? " " : "  ", v);
            s.append(b, (size_t)n);
        }
    });
    File f(path, "wb");
    if (!f.f) fail(UG4GB_ERR_INVALID, "%s: cannot open for writing (%s)", path, strerror(errno));
    f.write(head, path);
    for (auto &s : parts) f.write(s, path);
}

struct HostCsr {
    int rows = 0, cols = 0;
    std::vector<int> rp, ci;
    std::vector<double> va;
};

bool read_all(const char *path, std::string &s)
{
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    std::vector<char> buf(1 << 20);
    size_t n;
    while ((n = fread(buf.data(), 1, buf.size(), f)) > 0) s.append(buf.data(), n);
    fclose(f);
    return true;
}

// next line of s from position p (without the newline); false at the end
bool next_line(const std::string &s, size_t &p, const char *&b, const char *&e)
{
    if (p >= s.size()) return false;
    const size_t q = s.find('\n', p);
    b = s.data() + p;
    e = s.data() + (q == std::string::npos ? s.size() : q);
    p = (q == std::string::npos) ? s.size() : q + 1;
    if (e > b && e[-1] == '\r') --e;
    return true;
}

std::vector<std::string> words(const char *b, const char *e)
{
    std::vector<std::string> w;
    while (b < e) {
        while (b < e && (*b == ' ' || *b == '\t')) ++b;
        const char *s = b;
        while (b < e && *b != ' ' && *b != '\t') ++b;
        if (b > s) w.emplace_back(s, b);
    }
    return w;
}

// MatrixIOMtx(file, EXISTING) + read_into (matrix_io_mtx.h:202-236,
// matrix_io_mtx.cpp:170-268)
HostCsr mtx_read(const char *path)
{
    std::string s;
    if (!path || !read_all(path, s)) fail(UG4GB_ERR_INVALID, "File %s could not be found.", path ? path : "(null)");
    size_t p = 0;
    const char *b, *e;
    if (!next_line(s, p, b, e)) fail(UG4GB_ERR_INVALID, "%s: empty file", path);
    const std::vector<std::string> ban = words(b, e);
    if (ban.size() < 5 || ban[0] != "%%MatrixMarket" || ban[1] != "matrix")
        fail(UG4GB_ERR_INVALID, "%s: not a valid Matrix Market file (first line must start with "
                                "'%%%%MatrixMarket matrix')", path);
    if (ban[2] == "array") fail(UG4GB_ERR_INVALID, "Other than sparse MatrixMarket matrices are not yet implemented.");
    if (ban[2] != "coordinate") fail(UG4GB_ERR_INVALID, "MatrixMarket Type is invalid: %s", ban[2].c_str());
    if (ban[3] != "real" && ban[3] != "integer")
        fail(UG4GB_ERR_INVALID, "%s: MatrixMarket numeric type '%s' is not read (real and integer are)", path,
             ban[3].c_str());
    int kind;
    if (ban[4] == "general" || ban[4] == "hermitian") kind = MTX_GENERAL;   // hermitian: not mirrored, as ugcore
    else if (ban[4] == "symmetric") kind = MTX_SYMMETRIC;
    else if (ban[4] == "skew-symmetric") kind = MTX_SKEW;
    else fail(UG4GB_ERR_INVALID, "MatrixMarket algebraic type is invalid: %s", ban[4].c_str());

    // comment lines, then blank lines, then "rows cols lines"
    std::vector<std::string> dims;
    p = 0;
    while (true) {
        if (!next_line(s, p, b, e)) fail(UG4GB_ERR_INVALID, "%s: Unexpected end of file.", path);
        if (e > b && *b == '%') continue;
        dims = words(b, e);
        if (!dims.empty()) break;
    }
    if (dims.size() < 3) fail(UG4GB_ERR_INVALID, "%s: size line needs rows, columns and entries", path);
    char *end;
    const long long R = strtoll(dims[0].c_str(), &end, 10), C = strtoll(dims[1].c_str(), &end, 10),
                    L = strtoll(dims[2].c_str(), &end, 10);
    if (R < 0 || C < 0 || L < 0 || R > INT32_MAX || C > INT32_MAX)
        fail(UG4GB_ERR_INVALID, "%s: MatrixMarket matrix dimensions seem not be reasonable: (%lld, %lld, %lld)", path,
             R, C, L);

    // assignments in file order: (x, y) = v, then the mirrored one
    struct Asg {
        int64_t key;
        double v;
    };
    std::vector<Asg> asg;
    asg.reserve((size_t)L * (kind == MTX_GENERAL ? 1 : 2));
    for (long long i = 0; i < L; ++i) {
        if (!next_line(s, p, b, e)) fail(UG4GB_ERR_INVALID, "%s: %lld of %lld data lines found", path, i, L);
        std::string ln(b, e);
        const char *c0 = ln.c_str();
        char *c1, *c2, *c3;
        errno = 0;
        const long long x = strtoll(c0, &c1, 10);
        const long long y = strtoll(c1, &c2, 10);
        const double v = strtod(c2, &c3);
        if (c1 == c0 || c2 == c1 || c3 == c2)
            fail(UG4GB_ERR_INVALID, "Sparse matrix requires three values per line (%s, data line %lld)", path, i + 1);
        if (x < 1 || x > R || y < 1 || y > C)
            fail(UG4GB_ERR_INVALID, "%s: entry (%lld, %lld) outside the %lld x %lld matrix", path, x, y, R, C);
        asg.push_back({(x - 1) * C + (y - 1), v});
        if (kind != MTX_GENERAL && x != y) {
            if (y > R || x > C) fail(UG4GB_ERR_INVALID, "%s: mirrored entry (%lld, %lld) outside the matrix", path, y, x);
            asg.push_back({(y - 1) * C + (x - 1), kind == MTX_SYMMETRIC ? v : -v});
        }
    }
    std::stable_sort(asg.begin(), asg.end(), [](const Asg &a, const Asg &b) { return a.key < b.key; });
    HostCsr A;
    A.rows = (int)R;
    A.cols = (int)C;
    A.rp.assign((size_t)R + 1, 0);
    for (size_t a = 0; a < asg.size(); ++a) {
        if (a + 1 < asg.size() && asg[a + 1].key == asg[a].key) continue;   // a later assignment wins
        const int r = (int)(asg[a].key / C);
        A.ci.push_back((int)(asg[a].key % C));
        A.va.push_back(asg[a].v);
        ++A.rp[(size_t)r + 1];
    }
    for (int64_t r = 0; r < R; ++r) A.rp[r + 1] += A.rp[r];
    if (A.ci.size() > (size_t)INT32_MAX) fail(UG4GB_ERR_INVALID, "%s: too many entries", path);
    return A;
}

// --------------------------------------------------------- ConnectionViewer --
// WriteGridHeader (connection_viewer_output.h:95-112): version 1, dimension,
// N, one position per line ("%g"; 1D positions get a " 0.0"), then 1
std::string cv_header(int n, int dim, const double *pos)
{
    if (dim < 1 || dim > 3) fail(UG4GB_ERR_INVALID, "ConnectionViewer: dimension %d", dim);
    if (n > 0 && !pos) fail(UG4GB_ERR_INVALID, "ConnectionViewer: positions missing");
    std::string h;
    char b[160];
    h += "1\n";
    snprintf(b, sizeof b, "%d\n%d\n", dim, n);
    h += b;
    for (int i = 0; i < n; ++i) {
        const double *x = pos + (size_t)i * dim;
        if (dim == 1) snprintf(b, sizeof b, "%g 0.0\n", x[0]);
        else if (dim == 2) snprintf(b, sizeof b, "%g %g\n", x[0], x[1]);
        else snprintf(b, sizeof b, "%g %g %g\n", x[0], x[1], x[2]);
        h += b;
    }
    h += "1\n";
    return h;
}

void cv_write_matrix(int rows, const int *rp, const int *ci, const double *va, int dim, const double *pos,
                     const char *path)
{
    if (!path || !file_type_is(path, ".mat"))
        fail(UG4GB_ERR_INVALID, "Only '.mat' format supported for matrices, but filename is '%s'.",
             path ? path : "(null)");
    if (rows < 0 || !rp) fail(UG4GB_ERR_INVALID, "ConnectionViewer: bad matrix");
    const std::string head = cv_header(rows, dim, pos);
    const int T = num_threads();
    std::vector<std::string> parts(T);
    parallel_chunks(rows, 2048, [&](int t, int64_t lo, int64_t hi) {
        std::string &s = parts[t];
        char b[96];
        for (int64_t r = lo; r < hi; ++r)
            for (int a = rp[r]; a < rp[r + 1]; ++a) {
                const int n = (va[a] != 0.0) ? snprintf(b, sizeof b, "%lld %d %g\n", (long long)r, ci[a], va[a])
                                             : snprintf(b, sizeof b, "%lld %d 0\n", (long long)r, ci[a]);
                s.append(b, (size_t)n);
            }
    });
    File f(path, "wb");
    if (!f.f) fail(UG4GB_ERR_INVALID, "%s: cannot open for writing (%s)", path, strerror(errno));
    f.write(head, path);
    for (auto &s : parts) f.write(s, path);
}

void cv_write_vector(int n, const double *v, int dim, const double *pos, const char *path)
{
    if (!path || !file_type_is(path, ".vec"))
        fail(UG4GB_ERR_INVALID, "Only '.vec' format supported for vectors, but filename is '%s'.",
             path ? path : "(null)");
    if (n < 0 || (n > 0 && !v)) fail(UG4GB_ERR_INVALID, "ConnectionViewer: bad vector");
    const std::string head = cv_header(n, dim, pos);
    const int T = num_threads();
    std::vector<std::string> parts(T);
    parallel_chunks(n, 1 << 14, [&](int t, int64_t lo, int64_t hi) {
        std::string &s = parts[t];
        char b[96];
        for (int64_t i = lo; i < hi; ++i) {
            const int k = snprintf(b, sizeof b, "%lld %lld %.16g\n", (long long)i, (long long)i, v[i]);
            s.append(b, (size_t)k);
        }
    });
    File f(path, "wb");
    if (!f.f) fail(UG4GB_ERR_INVALID, "%s: cannot open for writing (%s)", path, strerror(errno));
    f.write(head, path);
    for (auto &s : parts) f.write(s, path);
}

// ReadVector (connection_viewer_input.h:104-150): header, positions skipped
// (two numbers each, three in 3D), then "from to value" triples until the end
// of the file or a trailing section that starts with 'c' or 'v'
void cv_read_vector(const char *path, int n, double *v)
{
    std::string s;
    if (!path || !read_all(path, s)) fail(UG4GB_ERR_INVALID, "Reading vector from %s failed.", path ? path : "(null)");
    const char *c = s.c_str();
    char *e;
    auto next_num = [&](const char *what) {
        const double x = strtod(c, &e);
        if (e == c) fail(UG4GB_ERR_INVALID, "%s: %s expected", path, what);
        c = e;
        return x;
    };
    const int version = (int)next_num("version"), dim = (int)next_num("dimension"), gridsize = (int)next_num("grid size");
    if (version != 1 || (dim != 2 && dim != 3) || gridsize < 0)
        fail(UG4GB_ERR_INVALID, "%s: header (version %d, dimension %d, size %d) not supported", path, version, dim,
             gridsize);
    if (gridsize != n) fail(UG4GB_ERR_INVALID, "%s: %d entries in the file, vector has %d", path, gridsize, n);
    for (int i = 0; i < gridsize; ++i)
        for (int k = 0; k < (dim == 3 ? 3 : 2); ++k) next_num("position");
    next_num("stringsInWindow flag");
    std::fill(v, v + n, 0.0);
    while (true) {
        while (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r') ++c;
        if (!*c || *c == 'c' || *c == 'v') break;
        const double from = next_num("index"), to = next_num("index"), val = next_num("value");
        if (from != to || from < 0 || from >= n || from != (double)(int64_t)from)
            fail(UG4GB_ERR_INVALID, "%s: bad entry index %g %g", path, from, to);
        v[(int64_t)from] = val;
    }
}

// -------------------------------------------------- device objects <-> host --
HostCsr export_matrix(const ug4gb_matrix *A)
{
    HostCsr h;
    int64_t nnz = 0;
    if (ug4gb_matrix_info(A, &h.rows, &h.cols, &nnz) != UG4GB_OK) fail(UG4GB_ERR_INVALID, "bad matrix");
    h.rp.resize((size_t)h.rows + 1);
    h.ci.resize((size_t)std::max<int64_t>(nnz, 1));
    h.va.resize((size_t)std::max<int64_t>(nnz, 1));
    const int rc = ug4gb_matrix_export_csr(A, h.rp.data(), h.ci.data(), h.va.data());
    if (rc != UG4GB_OK) fail(rc, "%s", ug4gb_last_error(A->ctx));
    return h;
}

std::vector<double> level_positions(const ug4gb_grid *g, int level, int &nv, int &dim)
{
    if (ug4gb_grid_level_info(g, level, &nv, nullptr, nullptr, &dim) != UG4GB_OK)
        fail(UG4GB_ERR_INVALID, "no such grid level %d", level);
    std::vector<double> pos((size_t)nv * dim);
    const int rc = ug4gb_grid_level_export(g, level, pos.data(), nullptr, nullptr);
    if (rc != UG4GB_OK) fail(rc, "%s", ug4gb_last_error(g->ctx));
    return pos;
}

template <class F>
int ctx_guarded(ug4gb_ctx *ctx, F &&f)
{
    char msg[512] = {0};
    const int rc = io_guarded(msg, sizeof msg, f);
    if (rc != UG4GB_OK && ctx) ctx->c.err = msg;
    return rc;
}

}  // namespace

extern "C" {

int ug4gb_io_write_mtx(int num_rows, int num_cols, const int *rowptr, const int *col, const double *val,
                       const char *filename, const char *comment, char *err, int err_capacity)
{
    return io_guarded(err, err_capacity, [&] { mtx_write(num_rows, num_cols, rowptr, col, val, filename, comment); });
}

int ug4gb_io_read_mtx_info(const char *filename, int *num_rows, int *num_cols, int64_t *nnz, char *err,
                           int err_capacity)
{
    return io_guarded(err, err_capacity, [&] {
        const HostCsr A = mtx_read(filename);
        if (num_rows) *num_rows = A.rows;
        if (num_cols) *num_cols = A.cols;
        if (nnz) *nnz = (int64_t)A.ci.size();
    });
}

int ug4gb_io_read_mtx(const char *filename, int *rowptr, int *col, double *val, char *err, int err_capacity)
{
    return io_guarded(err, err_capacity, [&] {
        const HostCsr A = mtx_read(filename);
        if (!rowptr || (!A.ci.empty() && (!col || !val))) fail(UG4GB_ERR_INVALID, "output arrays missing");
        std::copy(A.rp.begin(), A.rp.end(), rowptr);
        std::copy(A.ci.begin(), A.ci.end(), col);
        std::copy(A.va.begin(), A.va.end(), val);
    });
}

int ug4gb_io_write_cv_matrix(int num_rows, const int *rowptr, const int *col, const double *val, int dim,
                             const double *positions, const char *filename, char *err, int err_capacity)
{
    return io_guarded(err, err_capacity,
                      [&] { cv_write_matrix(num_rows, rowptr, col, val, dim, positions, filename); });
}

int ug4gb_io_write_cv_vector(int n, const double *values, int dim, const double *positions, const char *filename,
                             char *err, int err_capacity)
{
    return io_guarded(err, err_capacity, [&] { cv_write_vector(n, values, dim, positions, filename); });
}

int ug4gb_io_read_cv_vector(const char *filename, int n, double *values, char *err, int err_capacity)
{
    return io_guarded(err, err_capacity, [&] {
        if (n < 0 || (n > 0 && !values)) fail(UG4GB_ERR_INVALID, "output array missing");
        cv_read_vector(filename, n, values);
    });
}

int ug4gb_matrix_write_mtx(const ug4gb_matrix *A, const char *filename, const char *comment)
{
    if (!A) return UG4GB_ERR_INVALID;
    return ctx_guarded(A->ctx, [&] {
        const HostCsr h = export_matrix(A);
        mtx_write(h.rows, h.cols, h.rp.data(), h.ci.data(), h.va.data(), filename, comment);
    });
}

int ug4gb_matrix_read_mtx(ug4gb_matrix *A, const char *filename)
{
    if (!A) return UG4GB_ERR_INVALID;
    return ctx_guarded(A->ctx, [&] {
        const HostCsr h = mtx_read(filename);
        const int rc = ug4gb_matrix_set_csr(A, h.rows, h.cols, (int64_t)h.ci.size(), h.rp.data(),
                                            h.ci.empty() ? nullptr : h.ci.data(), h.va.empty() ? nullptr : h.va.data());
        if (rc != UG4GB_OK) fail(rc, "%s", ug4gb_last_error(A->ctx));
    });
}

int ug4gb_matrix_write_cv(const ug4gb_matrix *A, const ug4gb_grid *g, int level, const char *filename)
{
    if (!A || !g) return UG4GB_ERR_INVALID;
    return ctx_guarded(A->ctx, [&] {
        int nv, dim;
        const std::vector<double> pos = level_positions(g, level, nv, dim);
        const HostCsr h = export_matrix(A);
        if (h.rows != nv) fail(UG4GB_ERR_INVALID, "matrix has %d rows, grid level %d has %d vertices", h.rows, level, nv);
        cv_write_matrix(h.rows, h.rp.data(), h.ci.data(), h.va.data(), dim, pos.data(), filename);
    });
}

int ug4gb_vector_write_cv(const ug4gb_vector *v, const ug4gb_grid *g, int level, const char *filename)
{
    if (!v || !g) return UG4GB_ERR_INVALID;
    return ctx_guarded(v->ctx, [&] {
        int nv, dim;
        const std::vector<double> pos = level_positions(g, level, nv, dim);
        if (v->n != nv) fail(UG4GB_ERR_INVALID, "vector has %d entries, grid level %d has %d vertices", v->n, level, nv);
        std::vector<double> h((size_t)std::max(v->n, 1));
        const int rc = ug4gb_vector_copy_to(v, h.data());
        if (rc != UG4GB_OK) fail(rc, "%s", ug4gb_last_error(v->ctx));
        cv_write_vector(v->n, h.data(), dim, pos.data(), filename);
    });
}

int ug4gb_vector_read_cv(ug4gb_vector *v, const char *filename)
{
    if (!v) return UG4GB_ERR_INVALID;
    return ctx_guarded(v->ctx, [&] {
        std::vector<double> h((size_t)std::max(v->n, 1));
        cv_read_vector(filename, v->n, h.data());
        const int rc = ug4gb_vector_copy_from(v, h.data());
        if (rc != UG4GB_OK) fail(rc, "%s", ug4gb_last_error(v->ctx));
    });
}

}  // extern "C"
