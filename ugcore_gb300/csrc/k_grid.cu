// k_grid.cu -- structured hierarchy generation, CRS sparsity build, CRS
// transpose and CRS -> SELL-32 conversion.
//
// The CRS pattern of a level is the union of all element couplings with
// columns sorted per row and structural zeros kept: the set ugcore grows
// through SparseMatrix::operator()/get_index while adding element matrices
// (lib_algebra/cpu_algebra/sparsematrix_impl.h:553-701; AddLocalMatrixToGlobal,
// lib_disc/common/local_algebra.h:767).  It is built here without a global
// sort: vertex->element adjacency by counting, then one warp per row gathers
// the corners of its elements and ranks the distinct ones in shared memory.
#include <algorithm>

#include "common.cuh"

namespace ug4gb {

// ------------------------------------------------------------ generation --
__global__ void k_gen_vertices(int nx, int ny, int nz, int dim, double *coords, unsigned char *bnd,
                               int *color)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    int nv = nx * ny * nz;
    if (v >= nv) return;
    int i = v % nx, j = (v / nx) % ny, k = v / (nx * ny);
    coords[(size_t)v * dim + 0] = (double)i / (double)(nx - 1);
    coords[(size_t)v * dim + 1] = (double)j / (double)(ny - 1);
    int b = (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
    if (dim == 3) {
        coords[(size_t)v * dim + 2] = (double)k / (double)(nz - 1);
        b = b || (k == 0 || k == nz - 1);
    }
    bnd[v] = (unsigned char)b;
    color[v] = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
}

// quads: corners (i,j),(i+1,j),(i+1,j+1),(i,j+1); hexes: the reference
// hexahedron order; tets: 6 Kuhn tets per hex, orientation made positive.
__global__ void k_gen_elements(int elem_type, int nx, int ny, int nz, int *elems)
{
    int cx = nx - 1, cy = ny - 1, cz = (elem_type == UG4GB_QUAD) ? 1 : nz - 1;
    int ncell = cx * cy * cz;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int per = (elem_type == UG4GB_TET) ? 6 : 1;
    if (t >= ncell * per) return;
    int h = t / per, p = t % per;
    int i = h % cx, j = (h / cx) % cy, k = h / (cx * cy);
    int sx = 1, sy = nx, sz = nx * ny;
    int v0 = i + nx * (j + ny * k);
    if (elem_type == UG4GB_QUAD) {
        int *e = elems + 4 * (size_t)h;
        e[0] = v0; e[1] = v0 + 1; e[2] = v0 + 1 + nx; e[3] = v0 + nx;
    } else if (elem_type == UG4GB_HEX) {
        int *e = elems + 8 * (size_t)h;
        e[0] = v0; e[1] = v0 + sx; e[2] = v0 + sx + sy; e[3] = v0 + sy;
        e[4] = v0 + sz; e[5] = v0 + sx + sz; e[6] = v0 + sx + sy + sz; e[7] = v0 + sy + sz;
    } else {
        const int perm[6][2] = {{0, 1}, {0, 2}, {1, 0}, {1, 2}, {2, 0}, {2, 1}};
        int step[3] = {sx, sy, sz};
        int v1 = v0 + step[perm[p][0]], v2 = v1 + step[perm[p][1]], v3 = v0 + sx + sy + sz;
        bool odd = (p == 1 || p == 2 || p == 5);
        int *e = elems + 4 * (size_t)t;
        e[0] = v0; e[1] = odd ? v2 : v1; e[2] = odd ? v1 : v2; e[3] = v3;
    }
}

// parents of fine vertex (i,j,k) in the coarse level: vertex parent if all
// indices even; otherwise the corners of the coarse edge/face/cell
// (StdTransfer::assemble_prolongation_p1, std_transfer_impl.h:47-168), or for
// the Kuhn tet split the two ends of the coarse edge.
__global__ void k_gen_parents(int elem_type, int nx, int ny, int nz, int cnx, int cny, int *npar, int *par)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nx * ny * nz) return;
    int i = v % nx, j = (v / nx) % ny, k = v / (nx * ny);
    int p0 = i & 1, p1 = j & 1, p2 = k & 1;
    int b0 = i >> 1, b1 = j >> 1, b2 = k >> 1;
    int *out = par + 8 * (size_t)v;
    int n = 0;
    if (elem_type == UG4GB_TET) {
        out[n++] = b0 + cnx * (b1 + cny * b2);
        if (p0 | p1 | p2) out[n++] = (b0 + p0) + cnx * ((b1 + p1) + cny * (b2 + p2));
    } else {
        for (int dk = 0; dk <= p2; ++dk)
            for (int dj = 0; dj <= p1; ++dj)
                for (int di = 0; di <= p0; ++di) out[n++] = (b0 + di) + cnx * ((b1 + dj) + cny * (b2 + dk));
    }
    for (int q = n; q < 8; ++q) out[q] = -1;
    npar[v] = n;
}

void gen_level(Ctx &c, Level &L, int elem_type, int cx, int cy, int cz, const Level *coarse)
{
    L.elem_type = elem_type;
    L.dim = (elem_type == UG4GB_QUAD) ? 2 : 3;
    L.k = (elem_type == UG4GB_HEX) ? 8 : 4;
    L.nx = cx + 1; L.ny = cy + 1; L.nz = (L.dim == 3) ? cz + 1 : 1;
    L.nv = L.nx * L.ny * L.nz;
    int ncell = cx * cy * (L.dim == 3 ? cz : 1);
    L.ne = (elem_type == UG4GB_TET) ? 6 * ncell : ncell;
    L.coords.alloc((size_t)L.nv * L.dim);
    L.elems.alloc((size_t)L.ne * L.k);
    L.bnd.alloc(L.nv);
    L.color.alloc(L.nv);
    L.structured = true;
    L.ncolors = 1 << L.dim;
    UG_LAUNCH(c, k_gen_vertices, div_up(L.nv, 256), 256, 0, L.nx, L.ny, L.nz, L.dim, L.coords.p, L.bnd.p,
              L.color.p);
    UG_LAUNCH(c, k_gen_elements, div_up(L.ne, 256), 256, 0, elem_type, L.nx, L.ny, L.nz, L.elems.p);
    if (coarse) {
        L.npar.alloc(L.nv);
        L.par.alloc((size_t)L.nv * 8);
        UG_LAUNCH(c, k_gen_parents, div_up(L.nv, 256), 256, 0, elem_type, L.nx, L.ny, L.nz, coarse->nx, coarse->ny,
                  L.npar.p, L.par.p);
    }
}

// ----------------------------------------------------------------- scan --
// Exclusive scan of int32 (with int64 total): block-local scans, a single
// block scanning the block sums, then a fix-up pass.
constexpr int kScanBlock = 1024;

__global__ void k_scan_blocks(const int *in, int *out, int n, long long *block_sums)
{
    __shared__ long long sh[kScanBlock];
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    long long x = (i < n) ? in[i] : 0;
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        long long t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = (int)(sh[threadIdx.x] - x);
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void k_scan_sums(long long *block_sums, int nb, long long *total)
{
    // single block: sequential over chunks, parallel inside each
    __shared__ long long sh[kScanBlock];
    long long carry = 0;
    for (int base = 0; base < nb; base += kScanBlock) {
        int i = base + threadIdx.x;
        long long x = (i < nb) ? block_sums[i] : 0;
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            long long t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) block_sums[i] = carry + sh[threadIdx.x] - x;
        long long last = sh[kScanBlock - 1];
        __syncthreads();
        carry += last;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_fix(int *out, int n, const long long *block_sums)
{
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] = (int)(out[i] + block_sums[blockIdx.x]);
}

void exclusive_scan_int(Ctx &c, const int *in, int *out, int n, int64_t *total_out)
{
    int nb = (int)div_up(n > 0 ? n : 1, kScanBlock);
    DevBuf<long long> sums;
    sums.alloc(nb + 1);
    UG_LAUNCH(c, k_scan_blocks, nb, kScanBlock, 0, in, out, n, sums.p);
    UG_LAUNCH(c, k_scan_sums, 1, kScanBlock, 0, sums.p, nb, sums.p + nb);
    UG_LAUNCH(c, k_scan_fix, nb, kScanBlock, 0, out, n, sums.p);
    if (total_out) {
        long long t = 0;
        UG_CUDA(cudaMemcpyAsync(&t, sums.p + nb, sizeof(long long), cudaMemcpyDeviceToHost, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        *total_out = t;
    }
}

// ------------------------------------------------------- CRS from elems --
__global__ void k_count_corners(const int *elems, int nek, int *deg)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nek) atomicAdd(deg + elems[t], 1);
}

__global__ void k_fill_adjacency(const int *elems, int nek, int k, const int *vptr, int *cursor, int *adj)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nek) return;
    int v = elems[t];
    int pos = atomicAdd(cursor + v, 1);
    adj[vptr[v] + pos] = t / k;
}

constexpr int kRowCand = 256;   // max candidate columns per row (96 for Kuhn tets, 64 corner-sharing tets)

// One warp per row: gather corners of adjacent elements into shared memory,
// keep first occurrences, rank them.  mode 0 counts, mode 1 writes columns.
__global__ void k_row_pattern(const int *elems, int k, const int *vptr, const int *adj, int nv, int mode,
                              int *rowlen, const int *rowptr, int *col, int *overflow)
{
    __shared__ int cand[8][kRowCand];
    __shared__ int uniq[8][kRowCand];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * 8 + warp;
    if (row >= nv) return;
    int *cd = cand[warp], *uq = uniq[warp];
    const int a0 = vptr[row], a1 = vptr[row + 1];
    const int ncand = (a1 - a0) * k;
    if (ncand > kRowCand) {
        if (lane == 0) atomicExch(overflow, 1);
        return;
    }
    for (int t = lane; t < ncand; t += 32) cd[t] = elems[(size_t)adj[a0 + t / k] * k + (t % k)];
    __syncwarp();
    // keep the first occurrence of every column, mark repeats with INT_MAX
    for (int t = lane; t < ncand; t += 32) {
        int v = cd[t];
        bool first = true;
        for (int s = 0; s < t; ++s) first = first && (cd[s] != v);
        uq[t] = first ? v : 0x7fffffff;
    }
    __syncwarp();
    int nfirst_lane = 0;
    for (int t = lane; t < ncand; t += 32) {
        int v = uq[t];
        if (v == 0x7fffffff) continue;
        ++nfirst_lane;
        if (mode == 1) {
            int rank = 0;
            for (int s = 0; s < ncand; ++s) rank += (uq[s] < v) ? 1 : 0;
            col[rowptr[row] + rank] = v;
        }
    }
    if (mode == 0) {
        for (int o = 16; o > 0; o >>= 1) nfirst_lane += __shfl_xor_sync(0xffffffffu, nfirst_lane, o);
        if (lane == 0) rowlen[row] = nfirst_lane;
    }
}

void fill_double_impl(Ctx &c, double *p, size_t n, double v);

void csr_from_elements(Ctx &c, const Level &L, Csr &A)
{
    const int nv = L.nv, nek = L.ne * L.k;
    DevBuf<int> deg, vptr, cursor, adj, rowlen, overflow;
    deg.alloc(nv + 1);
    vptr.alloc(nv + 1);
    cursor.alloc(nv);
    adj.alloc(nek);
    rowlen.alloc(nv + 1);
    overflow.alloc(1);
    UG_CUDA(cudaMemsetAsync(deg.p, 0, deg.bytes(), c.stream));
    UG_CUDA(cudaMemsetAsync(cursor.p, 0, cursor.bytes(), c.stream));
    UG_CUDA(cudaMemsetAsync(overflow.p, 0, overflow.bytes(), c.stream));
    UG_LAUNCH(c, k_count_corners, div_up(nek, 256), 256, 0, L.elems.p, nek, deg.p);
    exclusive_scan_int(c, deg.p, vptr.p, nv + 1, nullptr);
    UG_LAUNCH(c, k_fill_adjacency, div_up(nek, 256), 256, 0, L.elems.p, nek, L.k, vptr.p, cursor.p, adj.p);
    UG_LAUNCH(c, k_row_pattern, div_up(nv, 8), 256, 0, L.elems.p, L.k, vptr.p, adj.p, nv, 0, rowlen.p,
              (const int *)nullptr, (int *)nullptr, overflow.p);
    UG_CUDA(cudaMemsetAsync(rowlen.p + nv, 0, sizeof(int), c.stream));
    A.nrows = A.ncols = nv;
    A.rowptr.alloc(nv + 1);
    int64_t nnz = 0;
    exclusive_scan_int(c, rowlen.p, A.rowptr.p, nv + 1, &nnz);
    int ovf = 0;
    UG_CUDA(cudaMemcpy(&ovf, overflow.p, sizeof(int), cudaMemcpyDeviceToHost));
    UG_REQUIRE(!ovf, UG4GB_ERR_INVALID, "csr_from_elements: a vertex couples to more than 256 element corners");
    UG_REQUIRE(nnz < (int64_t)1 << 31, UG4GB_ERR_INVALID, "csr_from_elements: nnz exceeds int32 range");
    A.nnz = nnz;
    A.col.alloc(nnz);
    A.val.alloc(nnz);
    UG_LAUNCH(c, k_row_pattern, div_up(nv, 8), 256, 0, L.elems.p, L.k, vptr.p, adj.p, nv, 1, (int *)nullptr,
              (const int *)A.rowptr.p, A.col.p, overflow.p);
    UG_CUDA(cudaMemsetAsync(A.val.p, 0, A.val.bytes(), c.stream));
}

// ------------------------------------------------------------ transpose --
__global__ void k_count_cols(const int *rowptr, const int *col, const double *val, int nrows, bool keep_zeros,
                             int *cnt)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a)
        if (keep_zeros || val[a] != 0.0) atomicAdd(cnt + col[a], 1);
}

__global__ void k_scatter_transpose(const int *rowptr, const int *col, const double *val, int nrows,
                                    bool keep_zeros, const int *trow, int *cursor, int *tcol, double *tval)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a) {
        if (!(keep_zeros || val[a] != 0.0)) continue;
        int cc = col[a];
        int pos = trow[cc] + atomicAdd(cursor + cc, 1);
        tcol[pos] = r;
        tval[pos] = val[a];
    }
}

// insertion sort of each (short) row by column
__global__ void k_sort_rows(const int *rowptr, int *col, double *val, int nrows)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    int a0 = rowptr[r], a1 = rowptr[r + 1];
    for (int a = a0 + 1; a < a1; ++a) {
        int cc = col[a];
        double vv = val[a];
        int b = a - 1;
        while (b >= a0 && col[b] > cc) {
            col[b + 1] = col[b];
            val[b + 1] = val[b];
            --b;
        }
        col[b + 1] = cc;
        val[b + 1] = vv;
    }
}

void csr_transpose(Ctx &c, const Csr &B, Csr &T, bool keep_zeros)
{
    T.nrows = B.ncols;
    T.ncols = B.nrows;
    DevBuf<int> cnt, cursor;
    cnt.alloc(T.nrows + 1);
    cursor.alloc(T.nrows + 1);
    UG_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), c.stream));
    UG_CUDA(cudaMemsetAsync(cursor.p, 0, cursor.bytes(), c.stream));
    UG_LAUNCH(c, k_count_cols, div_up(B.nrows, 256), 256, 0, B.rowptr.p, B.col.p, B.val.p, B.nrows, keep_zeros,
              cnt.p);
    T.rowptr.alloc(T.nrows + 1);
    int64_t nnz = 0;
    exclusive_scan_int(c, cnt.p, T.rowptr.p, T.nrows + 1, &nnz);
    T.nnz = nnz;
    T.col.alloc(nnz > 0 ? nnz : 1);
    T.val.alloc(nnz > 0 ? nnz : 1);
    UG_LAUNCH(c, k_scatter_transpose, div_up(B.nrows, 256), 256, 0, B.rowptr.p, B.col.p, B.val.p, B.nrows,
              keep_zeros, T.rowptr.p, cursor.p, T.col.p, T.val.p);
    UG_LAUNCH(c, k_sort_rows, div_up(T.nrows, 256), 256, 0, T.rowptr.p, T.col.p, T.val.p, T.nrows);
}

void csr_copy(Ctx &c, const Csr &src, Csr &dst)
{
    dst.nrows = src.nrows;
    dst.ncols = src.ncols;
    dst.nnz = src.nnz;
    dst.rowptr.alloc(src.nrows + 1);
    dst.col.alloc(src.nnz);
    dst.val.alloc(src.nnz);
    UG_CUDA(cudaMemcpyAsync(dst.rowptr.p, src.rowptr.p, src.rowptr.bytes(), cudaMemcpyDeviceToDevice, c.stream));
    if (src.nnz) {
        UG_CUDA(cudaMemcpyAsync(dst.col.p, src.col.p, (size_t)src.nnz * sizeof(int), cudaMemcpyDeviceToDevice,
                                c.stream));
        UG_CUDA(cudaMemcpyAsync(dst.val.p, src.val.p, (size_t)src.nnz * sizeof(double), cudaMemcpyDeviceToDevice,
                                c.stream));
    }
}

// ----------------------------------------------------------- CRS -> SELL --
__global__ void k_slice_width(const int *rowptr, int nrows, int nslices, int *w32)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslices) return;
    int w = 0;
    for (int r = s * kSliceH; r < min(nrows, (s + 1) * kSliceH); ++r) w = max(w, rowptr[r + 1] - rowptr[r]);
    w32[s] = w * kSliceH;
}

__global__ void k_slice_w_from32(const int *w32, int *w, int nslices)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nslices) w[s] = w32[s] / kSliceH;
}

template <class T>
__global__ void k_sell_fill(const int *rowptr, const int *col, const double *val, int nrows, const int *sptr,
                            const int *sw, const double *col_scale, int *scol, T *sval)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    int s = r / kSliceH, lane = r % kSliceH;
    if (s * kSliceH >= nrows) return;
    int w = sw[s];
    int base = sptr[s] + lane;
    int a0 = (r < nrows) ? rowptr[r] : 0, len = (r < nrows) ? rowptr[r + 1] - a0 : 0;
    int pad_col = (len > 0) ? col[a0 + len - 1] : 0;
    for (int q = 0; q < w; ++q) {
        int cc = pad_col;
        double v = 0.0;
        if (q < len) {
            cc = col[a0 + q];
            v = val[a0 + q];
            if (col_scale) v *= col_scale[cc];
        }
        scol[base + q * kSliceH] = cc;
        sval[base + q * kSliceH] = (T)v;
    }
}

template <class T>
void sell_from_csr(Ctx &c, const Csr &A, Sell<T> &S, const double *col_scale)
{
    S.nrows = A.nrows;
    S.ncols = A.ncols;
    S.nslices = (int)div_up(A.nrows > 0 ? A.nrows : 1, kSliceH);
    DevBuf<int> w32;
    w32.alloc(S.nslices + 1);
    S.sptr.alloc(S.nslices + 1);
    S.swidth.alloc(S.nslices);
    UG_CUDA(cudaMemsetAsync(w32.p, 0, w32.bytes(), c.stream));
    UG_LAUNCH(c, k_slice_width, div_up(S.nslices, 256), 256, 0, A.rowptr.p, A.nrows, S.nslices, w32.p);
    UG_LAUNCH(c, k_slice_w_from32, div_up(S.nslices, 256), 256, 0, w32.p, S.swidth.p, S.nslices);
    int64_t stored = 0;
    exclusive_scan_int(c, w32.p, S.sptr.p, S.nslices + 1, &stored);
    S.stored = stored;
    S.col.alloc(stored > 0 ? stored : 1);
    S.val.alloc(stored > 0 ? stored : 1);
    UG_LAUNCH(c, k_sell_fill<T>, div_up((size_t)S.nslices * kSliceH, 256), 256, 0, A.rowptr.p, A.col.p, A.val.p,
              A.nrows, S.sptr.p, S.swidth.p, col_scale, S.col.p, S.val.p);
}

template void sell_from_csr<double>(Ctx &, const Csr &, Sell<double> &, const double *);
template void sell_from_csr<float>(Ctx &, const Csr &, Sell<float> &, const double *);

// ------------------------------------------------------- CRS -> diagonal --
__global__ void k_offset_range(const int *rowptr, const int *col, int nrows, int *mn, int *mx)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    int lo = 0x7fffffff, hi = -0x7fffffff;
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a) {
        int o = col[a] - r;
        lo = min(lo, o);
        hi = max(hi, o);
    }
    if (rowptr[r + 1] > rowptr[r]) {
        atomicMin(mn, lo);
        atomicMax(mx, hi);
    }
}

__global__ void k_offset_mark(const int *rowptr, const int *col, int nrows, int lo, int *mark)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a) mark[col[a] - r - lo] = 1;
}

bool csr_offsets(Ctx &c, const Csr &A, int max_s, std::vector<int> &offs)
{
    offs.clear();
    if (A.nrows == 0 || A.nnz == 0) return false;
    DevBuf<int> mm;
    mm.alloc(2);
    int init[2] = {0x7fffffff, -0x7fffffff};
    UG_CUDA(cudaMemcpyAsync(mm.p, init, sizeof(init), cudaMemcpyHostToDevice, c.stream));
    UG_LAUNCH(c, k_offset_range, div_up(A.nrows, 256), 256, 0, A.rowptr.p, A.col.p, A.nrows, mm.p, mm.p + 1);
    int h[2];
    UG_CUDA(cudaMemcpyAsync(h, mm.p, sizeof(h), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    int64_t span = (int64_t)h[1] - h[0] + 1;
    if (span <= 0 || span > (int64_t)64 << 20) return false;
    DevBuf<int> mark;
    mark.alloc(span);
    UG_CUDA(cudaMemsetAsync(mark.p, 0, mark.bytes(), c.stream));
    UG_LAUNCH(c, k_offset_mark, div_up(A.nrows, 256), 256, 0, A.rowptr.p, A.col.p, A.nrows, h[0], mark.p);
    std::vector<int> hm(span);
    UG_CUDA(cudaMemcpyAsync(hm.data(), mark.p, mark.bytes(), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    for (int64_t i = 0; i < span; ++i)
        if (hm[i]) {
            offs.push_back((int)(i + h[0]));
            if ((int)offs.size() > max_s) return false;
        }
    return true;
}

template <class T>
__global__ void k_dia_fill(const int *rowptr, const int *col, const double *val, int nrows, int ld, Offs off, int S,
                           const double *col_scale, T *dval)
{
    PDL_ENTRY();
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a) {
        int o = col[a] - r;
        int k = 0;
        while (k < S && off.o[k] != o) ++k;
        if (k == S) continue;   // cannot happen: offs holds every offset of A
        double v = val[a];
        if (col_scale) v *= col_scale[col[a]];
        dval[(size_t)k * ld + r] = (T)v;
    }
}

// refill: D already holds this pattern's layout (the same offsets, the same
// CSR pattern): only the pattern's positions are rewritten, the zeros of the
// absent entries, the padding rows and the guards are kept
template <class T>
void dia_from_csr(Ctx &c, const Csr &A, Dia<T> &D, const std::vector<int> &offs, const double *col_scale,
                  bool refill)
{
    UG_REQUIRE((int)offs.size() <= kMaxDiag, UG4GB_ERR_INVALID, "dia_from_csr: too many offsets");
    const size_t want = (size_t)offs.size() * ((A.nrows + 31) / 32 * 32) + 2 * Dia<T>::kGuard;
    refill = refill && D.val.p && D.val.n == want && D.S == (int)offs.size() && D.nrows == A.nrows;
    D.nrows = A.nrows;
    D.ncols = A.ncols;
    D.S = (int)offs.size();
    for (int k = 0; k < kMaxDiag; ++k) D.off.o[k] = k < D.S ? offs[k] : 0;
    D.ld = (A.nrows + 31) / 32 * 32;
    D.val.alloc((size_t)D.S * D.ld + 2 * Dia<T>::kGuard);
    // absent entries, the padding rows and the guards stay 0
    if (!refill) UG_CUDA(cudaMemsetAsync(D.val.p, 0, D.val.bytes(), c.stream));
    UG_LAUNCH_PDL(c, k_dia_fill<T>, div_up(A.nrows, 256), 256, 0, A.rowptr.p, A.col.p, A.val.p, A.nrows, D.ld, D.off,
              D.S, col_scale, D.vals());
}

// the diagonal kernels are instantiated for S = 9, 15, 27 (2D quads, Kuhn
// tets, hexahedra); a smaller offset set is padded with offset 0 (value 0)
static int dia_width(int s)
{
    if (s <= 9) return 9;
    if (s <= 15) return 15;
    if (s <= 27) return 27;
    return 0;
}

template <class T>
void op_from_csr(Ctx &c, const Csr &A, OpMat<T> &M, const double *col_scale, bool allow_dia)
{
    M.nrows = A.nrows;
    M.ncols = A.ncols;
    std::vector<int> offs;
    if (allow_dia && A.nrows == A.ncols && csr_offsets(c, A, 27, offs)) {
        int w = dia_width((int)offs.size());
        // pad with offsets that do not occur (value 0), keeping the set sorted
        int cand = 1;
        while ((int)offs.size() < w) {
            bool have = false;
            for (int o : offs) have = have || (o == cand);
            if (!have) offs.push_back(cand);
            cand = (cand > 0) ? -cand : -cand + 1;
        }
        std::sort(offs.begin(), offs.end());
        M.kind = 1;
        dia_from_csr<T>(c, A, M.dia, offs, col_scale);
        M.sell = Sell<T>();
    } else {
        M.kind = 0;
        sell_from_csr<T>(c, A, M.sell, col_scale);
        M.dia = Dia<T>();
    }
}

template <class T>
void op_from_csr_cached(Ctx &c, const Csr &A, OpMat<T> &M, const double *col_scale, bool allow_dia, OpLayout &lay)
{
    if (lay.known && lay.nrows == A.nrows && lay.nnz == A.nnz && (lay.kind == 0 || allow_dia)) {
        if (lay.kind == 1) {
            dia_from_csr<T>(c, A, M.dia, lay.offs, col_scale, M.kind == 1);
        } else {
            UG_LAUNCH(c, k_sell_fill<T>, div_up((size_t)M.sell.nslices * kSliceH, 256), 256, 0, A.rowptr.p, A.col.p,
                      A.val.p, A.nrows, M.sell.sptr.p, M.sell.swidth.p, col_scale, M.sell.col.p, M.sell.val.p);
        }
        return;
    }
    op_from_csr<T>(c, A, M, col_scale, allow_dia);
    lay.known = true;
    lay.kind = M.kind;
    lay.nrows = A.nrows;
    lay.nnz = A.nnz;
    lay.offs.assign(M.dia.off.o, M.dia.off.o + (M.kind == 1 ? M.dia.S : 0));
}

template void op_from_csr_cached<double>(Ctx &, const Csr &, OpMat<double> &, const double *, bool, OpLayout &);
template void op_from_csr_cached<float>(Ctx &, const Csr &, OpMat<float> &, const double *, bool, OpLayout &);

__global__ void k_iota_val(double *v, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (double)i;
}

// perm from the transposed index values; then the real values through it
__global__ void k_perm_gather(int64_t n, const double *tidx, int *perm, const double *aval, double *tval)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int a = (int)tidx[k];
    perm[k] = a;
    tval[k] = aval[a];
}

__global__ void k_gather_perm(int64_t n, const int *perm, const double *aval, double *tval)
{
    PDL_ENTRY();
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) tval[k] = aval[perm[k]];
}

void transpose_perm(Ctx &c, const Csr &A, Csr &T, DevBuf<int> &perm)
{
    UG_REQUIRE(A.nnz < ((int64_t)1 << 31), UG4GB_ERR_INVALID, "transpose_perm: nnz exceeds int32 range");
    Csr B;
    B.nrows = A.nrows;
    B.ncols = A.ncols;
    B.nnz = A.nnz;
    B.rowptr.alloc(A.nrows + 1);
    B.col.alloc(A.nnz > 0 ? A.nnz : 1);
    B.val.alloc(A.nnz > 0 ? A.nnz : 1);
    UG_CUDA(cudaMemcpyAsync(B.rowptr.p, A.rowptr.p, sizeof(int) * (size_t)(A.nrows + 1), cudaMemcpyDeviceToDevice,
                            c.stream));
    if (A.nnz) {
        UG_CUDA(cudaMemcpyAsync(B.col.p, A.col.p, sizeof(int) * (size_t)A.nnz, cudaMemcpyDeviceToDevice, c.stream));
        UG_LAUNCH(c, k_iota_val, div_up(A.nnz, (int64_t)256), 256, 0, B.val.p, A.nnz);
    }
    csr_transpose(c, B, T, true);
    perm.alloc(T.nnz > 0 ? T.nnz : 1);
    if (T.nnz) {
        DevBuf<double> tidx;
        tidx.alloc(T.nnz);
        UG_CUDA(cudaMemcpyAsync(tidx.p, T.val.p, sizeof(double) * (size_t)T.nnz, cudaMemcpyDeviceToDevice, c.stream));
        UG_LAUNCH(c, k_perm_gather, div_up(T.nnz, (int64_t)256), 256, 0, T.nnz, tidx.p, perm.p, A.val.p, T.val.p);
        UG_CUDA(cudaStreamSynchronize(c.stream));
    }
}

__global__ void k_diff_int(int64_t n, const int *a, const int *b, int *flag)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && a[i] != b[i]) *flag = 1;
}

bool csr_same_pattern(Ctx &c, const Csr &A, const Csr &B)
{
    if (A.nrows != B.nrows || A.ncols != B.ncols || A.nnz != B.nnz) return false;
    DevBuf<int> flag;
    flag.alloc(1);
    UG_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c.stream));
    UG_LAUNCH(c, k_diff_int, div_up((int64_t)A.nrows + 1, (int64_t)256), 256, 0, (int64_t)A.nrows + 1, A.rowptr.p,
              B.rowptr.p, flag.p);
    if (A.nnz) UG_LAUNCH(c, k_diff_int, div_up(A.nnz, (int64_t)256), 256, 0, A.nnz, A.col.p, B.col.p, flag.p);
    int h = 0;
    UG_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    return h == 0;
}

// position of column c in row r (columns sorted), or -1
__device__ __forceinline__ int row_find(const int *__restrict__ rowptr, const int *__restrict__ col, int r, int c)
{
    int lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int cm = col[mid];
        if (cm == c) return mid;
        if (cm < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

__global__ void k_check_symmetric(const int *rowptr, const int *col, int n, int *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int a = rowptr[i]; a < rowptr[i + 1]; ++a) {
        const int j = col[a];
        if (j != i && (j < 0 || j >= n || row_find(rowptr, col, j, i) < 0)) {
            atomicExch(bad, 1);
            return;
        }
    }
}

// entry (i, j) swapped with (j, i), each pair by the row with the smaller index
__global__ void k_transpose_symmetric(const int *rowptr, const int *col, double *val, int n)
{
    PDL_ENTRY();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int a = rowptr[i]; a < rowptr[i + 1]; ++a) {
        const int j = col[a];
        if (j <= i) continue;
        const int b = row_find(rowptr, col, j, i);
        if (b < 0) continue;
        const double t = val[a];
        val[a] = val[b];
        val[b] = t;
    }
}

bool csr_pattern_symmetric(Ctx &c, const Csr &A)
{
    if (A.nrows != A.ncols) return false;
    if (A.nrows == 0) return true;
    DevBuf<int> bad;
    bad.alloc(1);
    UG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), c.stream));
    UG_LAUNCH(c, k_check_symmetric, div_up(A.nrows, 256), 256, 0, A.rowptr.p, A.col.p, A.nrows, bad.p);
    int h = 0;
    UG_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    return h == 0;
}

void csr_transpose_symmetric_inplace(Ctx &c, Csr &A)
{
    if (A.nrows) UG_LAUNCH_PDL(c, k_transpose_symmetric, div_up(A.nrows, 256), 256, 0, A.rowptr.p, A.col.p, A.val.p, A.nrows);
}

void transpose_values(Ctx &c, const Csr &A, Csr &T, const DevBuf<int> &perm)
{
    if (T.nnz) UG_LAUNCH_PDL(c, k_gather_perm, div_up(T.nnz, (int64_t)256), 256, 0, T.nnz, perm.p, A.val.p, T.val.p);
}

template void dia_from_csr<double>(Ctx &, const Csr &, Dia<double> &, const std::vector<int> &, const double *,
                                   bool);
template void dia_from_csr<float>(Ctx &, const Csr &, Dia<float> &, const std::vector<int> &, const double *,
                                  bool);
template void op_from_csr<double>(Ctx &, const Csr &, OpMat<double> &, const double *, bool);
template void op_from_csr<float>(Ctx &, const Csr &, OpMat<float> &, const double *, bool);

__global__ void k_fill(double *p, size_t n, double v)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

void fill_double(Ctx &c, double *p, size_t n, double v)
{
    if (n == 0) return;
    UG_LAUNCH(c, k_fill, div_up(n, 256), 256, 0, p, n, v);
}

void check_device_error(Ctx &c)
{
    if (!c.dev_err.p || !c.dev_err_possible) return;
    int flag = 0;
    UG_CUDA(cudaMemcpy(&flag, c.dev_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        UG_CUDA(cudaMemset(c.dev_err.p, 0, sizeof(int)));
        throw Error{UG4GB_ERR_CUDA, "a kernel's bounded wait for its own asynchronous copies ran out"};
    }
}

}  // namespace ug4gb
