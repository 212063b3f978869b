// sparse_matrix_t: the reference's spmv.h API (spmv/spmv.h:11-84) over host
// layouts built by layout.cpp, with the products on the GPU.
//
// Three device variants of y = op(A) x:
//   SELL  warp-sliced ELL over rows sorted by length (1 to 32 lanes per
//         row, 1 or 4 entries per lane per step);
//   BLOCK the reference's 4-row block arena, uploaded byte for byte, one
//         quad of lanes per block (spmv_block.c:160-254);
//   CSR   sub-warp per row over the reference's CSR arrays, shuffle sums.
// SELL and BLOCK add each row's products in the reference's order with
// separate rounding of products and sums, so their results are
// bit-identical to the reference's block product; CSR re-associates.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/acdalm_ext.h"
#include "../../include/spmv.h"
#include "common.h"
#include "device.cuh"
#include "layout.h"

namespace acd {

// Grid-stride warps over a whole (non-cooperative) launch; x is read-only.
// The matrix is streamed once per product, so its loads are tagged
// evict-first in L2 and the gathered x keeps its lines.
struct FlatTeam {
        static constexpr bool kStreamHint = true;
        unsigned long long policy = evict_first_policy();
        __device__ int nthreads() const { return gridDim.x * blockDim.x; }
        __device__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
        __device__ int warp() const { return tid() >> 5; }
        __device__ int nwarps() const { return nthreads() >> 5; }
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return __ldg(p); }
};

template <class T, bool Exact>
__global__ void sell_kernel(SellDev<T> op, const int32_t * row_of_d,
                            const T * x, T * y)
{
        FlatTeam tm;
        sell_rows_1<Exact>(tm, op, x, [&](int d, T acc) { y[row_of_d[d]] = acc; });
}

template <class T, bool Exact>
__global__ void sell2_kernel(SellDev<T> op, const int32_t * row_of_d,
                             const T * x0, const T * x1, T * y0, T * y1)
{
        FlatTeam tm;
        sell_rows_2<Exact>(tm, op, x0, x1, [&](int d, T a0, T a1) {
                int r = row_of_d[d];
                y0[r] = a0;
                y1[r] = a1;
        });
}

// The reference's block arena: header {u32 width, u32 start_row, u32 rows}
// padded to 32 bytes, width x double[4] slot values, width x u32[4] columns.
template <class T>
__global__ void block4_kernel(const uint8_t * arena, const size_t * offsets,
                              int nblocks, const double * x0, const double * x1,
                              double * y0, double * y1)
{
        int gt = blockIdx.x * blockDim.x + threadIdx.x;
        int r = gt & 3;
        for (int b = gt >> 2; b < nblocks; b += (gridDim.x * blockDim.x) >> 2) {
                const uint8_t * base = arena + offsets[b];
                const uint32_t * hdr = reinterpret_cast<const uint32_t *>(base);
                int width = (int)__ldg(hdr), start = (int)__ldg(hdr + 1),
                    nr = (int)__ldg(hdr + 2);
                const double * vals = reinterpret_cast<const double *>(base + 32);
                const uint32_t * cols = reinterpret_cast<const uint32_t *>(vals + 4 * width);
                double a0 = 0, a1 = 0;
                for (int s = 0; s < width; s++) {
                        double v = __ldg(vals + 4 * s + r);
                        uint32_t c = __ldg(cols + 4 * s + r);
                        a0 = __dadd_rn(a0, __dmul_rn(v, __ldg(x0 + c)));
                        if (x1)
                                a1 = __dadd_rn(a1, __dmul_rn(v, __ldg(x1 + c)));
                }
                if (r < nr) {
                        y0[start + r] = a0;
                        if (y1)
                                y1[start + r] = a1;
                }
        }
}

// CSR with SUB lanes per row; each lane takes every SUB-th entry, then a
// shuffle tree sums the lanes.
template <class T, int SUB>
__global__ void csr_kernel(const uint32_t * ptr, const uint32_t * col,
                           const T * val, int nrows, const T * x0, const T * x1,
                           T * y0, T * y1)
{
        constexpr int kRows = 32 / SUB;  // rows per warp per step
        int gt = blockIdx.x * blockDim.x + threadIdx.x;
        int sl = threadIdx.x % SUB;
        int sub_id = (threadIdx.x & 31) / SUB;
        int nwarps = (gridDim.x * blockDim.x) >> 5;
        // the loop bound is uniform across the warp, so every lane reaches
        // the shuffles
        for (int base = (gt >> 5) * kRows; base < nrows; base += nwarps * kRows) {
                int row = base + sub_id;
                T a0 = 0, a1 = 0;
                if (row < nrows) {
                        uint32_t b = __ldg(ptr + row), e = __ldg(ptr + row + 1);
                        for (uint32_t j = b + sl; j < e; j += SUB) {
                                T v = __ldg(val + j);
                                uint32_t c = __ldg(col + j);
                                a0 += v * __ldg(x0 + c);
                                if (x1)
                                        a1 += v * __ldg(x1 + c);
                        }
                }
#pragma unroll
                for (int o = SUB / 2; o > 0; o >>= 1) {
                        a0 += __shfl_down_sync(0xffffffffu, a0, o, SUB);
                        if (x1)
                                a1 += __shfl_down_sync(0xffffffffu, a1, o, SUB);
                }
                if (sl == 0 && row < nrows) {
                        y0[row] = a0;
                        if (y1)
                                y1[row] = a1;
                }
        }
}

}  // namespace acd

// ---------------------------------------------------------------------------

struct DevSpmvLayout {
        bool ready = false;
        void * mem = nullptr;
        size_t bytes = 0;
        // SELL
        acd::SellDev<double> sell{};
        acd::SellDev<float> sellf{};
        int32_t * row_of_d = nullptr;
        float * valf = nullptr;
        // BLOCK
        uint8_t * arena = nullptr;
        size_t * offsets = nullptr;
        int nblocks = 0;
        // CSR
        uint32_t * ptr = nullptr;
        uint32_t * col = nullptr;
        double * val = nullptr;
        float * csr_valf = nullptr;
        int nrows = 0;
        double mean_len = 0;
};

struct sparse_matrix {
        acd::HostMatrix h;
        std::mutex lock;
        DevSpmvLayout dev[3][2];  // [variant][transpose]
        cudaStream_t stream = nullptr;
        double * scratch = nullptr;  // 4 * max(m, n) doubles for host calls
        size_t scratch_len = 0;
};

namespace {

int g_variant = ACDALM_SPMV_SELL;

template <class T>
T * carve(char *& p, size_t count)
{
        T * r = reinterpret_cast<T *>(p);
        p += (count * sizeof(T) + 255) & ~size_t(255);
        return r;
}

size_t rnd(size_t b)
{
        return (b + 255) & ~size_t(255);
}

int ensure_stream(sparse_matrix_t * a)
{
        if (a->stream)
                return 0;
        if (!acd::device_ready())
                return ACDALM_ENODEV;
        ACD_CUDA_TRY(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking),
                     ACDALM_ECUDA);
        return 0;
}

int ensure_layout(sparse_matrix_t * a, int variant, int transpose, bool f32)
{
        DevSpmvLayout & L = a->dev[variant][transpose];
        int r = ensure_stream(a);
        if (r)
                return r;
        if (!L.ready) {
                const acd::Csr & c = transpose ? a->h.csr_t : a->h.csr;
                L.nrows = (int)c.nrows;
                L.mean_len = c.nrows ? (double)a->h.nnz / c.nrows : 0;
                if (variant == ACDALM_SPMV_SELL) {
                        acd::PlainSell ps;
                        acd::build_plain_sell(a->h, transpose, ps);
                        size_t e = ps.s.ptr.back();
                        size_t ns = std::max<size_t>(ps.s.row0.size(), 1);
                        size_t total = rnd(ps.s.ptr.size() * 8) + rnd(ns * 4) + rnd(e * 4)
                                + rnd(e * 8) + rnd(e * 4)
                                + rnd(std::max<size_t>(ps.row_of_d.size(), 1) * 4);
                        ACD_CUDA_TRY(cudaMalloc(&L.mem, total), ACDALM_ENOMEM);
                        L.bytes = total;
                        char * p = static_cast<char *>(L.mem);
                        int64_t * dptr = carve<int64_t>(p, ps.s.ptr.size());
                        int32_t * drow0 = carve<int32_t>(p, ns);
                        int32_t * dcol = carve<int32_t>(p, e);
                        double * dval = carve<double>(p, e);
                        L.valf = carve<float>(p, e);
                        L.row_of_d = carve<int32_t>(p, std::max<size_t>(ps.row_of_d.size(), 1));
                        std::vector<float> vf(ps.s.val.begin(), ps.s.val.end());
                        ACD_CUDA_TRY(cudaMemcpy(dptr, ps.s.ptr.data(), ps.s.ptr.size() * 8,
                                                cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        if (!ps.s.row0.empty())
                                ACD_CUDA_TRY(cudaMemcpy(drow0, ps.s.row0.data(), ps.s.row0.size() * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        if (e) {
                                ACD_CUDA_TRY(cudaMemcpy(dcol, ps.s.col.data(), e * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                                ACD_CUDA_TRY(cudaMemcpy(dval, ps.s.val.data(), e * 8,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                                ACD_CUDA_TRY(cudaMemcpy(L.valf, vf.data(), e * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        }
                        if (!ps.row_of_d.empty())
                                ACD_CUDA_TRY(cudaMemcpy(L.row_of_d, ps.row_of_d.data(),
                                                        ps.row_of_d.size() * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        L.sell = {ps.s.nrows, ps.s.nslices, dptr, drow0, dcol, dval};
                        L.sellf = {ps.s.nrows, ps.s.nslices, dptr, drow0, dcol, L.valf};
                } else if (variant == ACDALM_SPMV_BLOCK) {
                        acd::ensure_blocks(a->h);
                        const acd::BlockArena & B = transpose ? a->h.block_t : a->h.block;
                        size_t total = rnd(std::max<size_t>(B.bytes.size(), 1))
                                + rnd(std::max<size_t>(B.nblocks, 1) * 8);
                        ACD_CUDA_TRY(cudaMalloc(&L.mem, total), ACDALM_ENOMEM);
                        L.bytes = total;
                        char * p = static_cast<char *>(L.mem);
                        L.arena = carve<uint8_t>(p, std::max<size_t>(B.bytes.size(), 1));
                        L.offsets = carve<size_t>(p, std::max<size_t>(B.nblocks, 1));
                        L.nblocks = (int)B.nblocks;
                        if (!B.bytes.empty())
                                ACD_CUDA_TRY(cudaMemcpy(L.arena, B.bytes.data(), B.bytes.size(),
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        if (B.nblocks)
                                ACD_CUDA_TRY(cudaMemcpy(L.offsets, B.offsets.data(), B.nblocks * 8,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                } else {
                        size_t nnz = a->h.nnz;
                        size_t total = rnd((c.nrows + 1) * 4) + rnd(std::max<size_t>(nnz, 1) * 4)
                                + rnd(std::max<size_t>(nnz, 1) * 8) + rnd(std::max<size_t>(nnz, 1) * 4);
                        ACD_CUDA_TRY(cudaMalloc(&L.mem, total), ACDALM_ENOMEM);
                        L.bytes = total;
                        char * p = static_cast<char *>(L.mem);
                        L.ptr = carve<uint32_t>(p, c.nrows + 1);
                        L.col = carve<uint32_t>(p, std::max<size_t>(nnz, 1));
                        L.val = carve<double>(p, std::max<size_t>(nnz, 1));
                        L.csr_valf = carve<float>(p, std::max<size_t>(nnz, 1));
                        std::vector<float> vf(c.val.begin(), c.val.end());
                        ACD_CUDA_TRY(cudaMemcpy(L.ptr, c.ptr.data(), (c.nrows + 1) * 4,
                                                cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        if (nnz) {
                                ACD_CUDA_TRY(cudaMemcpy(L.col, c.col.data(), nnz * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                                ACD_CUDA_TRY(cudaMemcpy(L.val, c.val.data(), nnz * 8,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                                ACD_CUDA_TRY(cudaMemcpy(L.csr_valf, vf.data(), nnz * 4,
                                                        cudaMemcpyHostToDevice), ACDALM_ECUDA);
                        }
                }
                L.ready = true;
        }
        (void)f32;
        return 0;
}

int grid_for(long long units, int per_block)
{
        long long b = (units + per_block - 1) / per_block;
        return (int)std::max(1LL, std::min(b, 152LL * 16));
}

template <class T>
int launch(sparse_matrix_t * a, int variant, int transpose, const T * x0,
           const T * x1, T * y0, T * y1, cudaStream_t s)
{
        bool f32 = sizeof(T) == 4;
        // the fused-rounding SELL product runs over the SELL layout
        bool fused = variant == ACDALM_SPMV_SELL_FMA;
        if (fused)
                variant = ACDALM_SPMV_SELL;
        int r = ensure_layout(a, variant, transpose, f32);
        if (r)
                return r;
        DevSpmvLayout & L = a->dev[variant][transpose];
        if (L.nrows == 0)
                return 0;
        if (variant == ACDALM_SPMV_SELL) {
                int blocks = grid_for((long long)L.sell.nslices * 32, 256);
                if constexpr (sizeof(T) == 8) {
                        if (fused) {
                                if (x1)
                                        acd::sell2_kernel<double, false><<<blocks, 256, 0, s>>>(
                                                L.sell, L.row_of_d, x0, x1, y0, y1);
                                else
                                        acd::sell_kernel<double, false><<<blocks, 256, 0, s>>>(
                                                L.sell, L.row_of_d, x0, y0);
                        } else if (x1) {
                                acd::sell2_kernel<double, true><<<blocks, 256, 0, s>>>(
                                        L.sell, L.row_of_d, x0, x1, y0, y1);
                        } else {
                                acd::sell_kernel<double, true><<<blocks, 256, 0, s>>>(
                                        L.sell, L.row_of_d, x0, y0);
                        }
                } else {
                        if (x1)
                                acd::sell2_kernel<float, false><<<blocks, 256, 0, s>>>(
                                        L.sellf, L.row_of_d, x0, x1, y0, y1);
                        else
                                acd::sell_kernel<float, false><<<blocks, 256, 0, s>>>(
                                        L.sellf, L.row_of_d, x0, y0);
                }
        } else if (variant == ACDALM_SPMV_BLOCK) {
                if constexpr (sizeof(T) == 8) {
                        int blocks = grid_for((long long)L.nblocks * 4, 256);
                        acd::block4_kernel<double><<<blocks, 256, 0, s>>>(
                                L.arena, L.offsets, L.nblocks, x0, x1, y0, y1);
                } else {
                        acd::set_error(ACDALM_EINVAL, "the block variant is FP64 only");
                        return ACDALM_EINVAL;
                }
        } else {
                int sub = L.mean_len > 24 ? 32 : L.mean_len > 12 ? 16 : L.mean_len > 6 ? 8 : 4;
                const T * val;
                if constexpr (sizeof(T) == 8)
                        val = L.val;
                else
                        val = L.csr_valf;
                int blocks = grid_for((long long)L.nrows * sub, 256);
#define ACD_CSR(S)                                                                   \
        acd::csr_kernel<T, S><<<blocks, 256, 0, s>>>(L.ptr, L.col, val, L.nrows, x0, \
                                                     x1, y0, y1)
                if (sub == 32)
                        ACD_CSR(32);
                else if (sub == 16)
                        ACD_CSR(16);
                else if (sub == 8)
                        ACD_CSR(8);
                else
                        ACD_CSR(4);
#undef ACD_CSR
        }
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        acd::count_launch();
        return 0;
}

int host_multiply(double ** y, size_t ny, const sparse_matrix_t * ca,
                  const double ** x, size_t nx, int transpose, int nrhs)
{
        sparse_matrix_t * a = const_cast<sparse_matrix_t *>(ca);
        size_t nrows = transpose ? a->h.ncols : a->h.nrows;
        size_t ncols = transpose ? a->h.nrows : a->h.ncols;
        if (ny != nrows || nx != ncols) {
                acd::set_error(ACDALM_EINVAL, "sparse_matrix_multiply: %zu x %zu operator, "
                               "ny = %zu, nx = %zu", nrows, ncols, ny, nx);
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(a->lock);
        int r = ensure_stream(a);
        if (r)
                return r;
        size_t len = std::max<size_t>(std::max(a->h.nrows, a->h.ncols), 1);
        if (a->scratch_len < len) {
                if (a->scratch)
                        cudaFree(a->scratch);
                a->scratch = nullptr;
                ACD_CUDA_TRY(cudaMalloc(&a->scratch, 4 * len * sizeof(double)), ACDALM_ENOMEM);
                a->scratch_len = len;
        }
        double * dx0 = a->scratch, * dx1 = a->scratch + len;
        double * dy0 = a->scratch + 2 * len, * dy1 = a->scratch + 3 * len;
        cudaStream_t s = a->stream;
        if (nx) {
                ACD_CUDA_TRY(cudaMemcpyAsync(dx0, x[0], nx * 8, cudaMemcpyHostToDevice, s),
                             ACDALM_ECUDA);
                if (nrhs == 2)
                        ACD_CUDA_TRY(cudaMemcpyAsync(dx1, x[1], nx * 8, cudaMemcpyHostToDevice, s),
                                     ACDALM_ECUDA);
        }
        if (ny) {
                // empty rows are written too (their sum is 0)
                r = launch<double>(a, g_variant, transpose, dx0, nrhs == 2 ? dx1 : nullptr,
                                   dy0, nrhs == 2 ? dy1 : nullptr, s);
                if (r)
                        return r;
                ACD_CUDA_TRY(cudaMemcpyAsync(y[0], dy0, ny * 8, cudaMemcpyDeviceToHost, s),
                             ACDALM_ECUDA);
                if (nrhs == 2)
                        ACD_CUDA_TRY(cudaMemcpyAsync(y[1], dy1, ny * 8, cudaMemcpyDeviceToHost, s),
                                     ACDALM_ECUDA);
        }
        ACD_CUDA_TRY(cudaStreamSynchronize(s), ACDALM_ECUDA);
        return 0;
}

}  // namespace

extern "C" {

void sparse_matrix_init(void)
{
        acd::device_ready();
}

sparse_matrix_t * sparse_matrix_make(size_t ncolumns, size_t nrows, size_t nnz,
                                     const uint32_t * rows, const uint32_t * columns,
                                     const double * values, int permute)
{
        if ((nnz && (!rows || !columns || !values)) || nrows >= (1ull << 31)
            || ncolumns >= (1ull << 31) || nnz >= (1ull << 32)) {
                acd::set_error(ACDALM_EINVAL, "sparse_matrix_make: bad arguments");
                return nullptr;
        }
        for (size_t i = 0; i < nnz; i++)
                if (rows[i] >= nrows || columns[i] >= ncolumns) {
                        acd::set_error(ACDALM_EINVAL,
                                       "sparse_matrix_make: entry %zu at (%u, %u) is outside "
                                       "the %zu x %zu matrix", i, rows[i], columns[i], nrows,
                                       ncolumns);
                        return nullptr;
                }
        sparse_matrix_t * m = new (std::nothrow) sparse_matrix;
        if (!m) {
                acd::set_error(ACDALM_ENOMEM, "sparse_matrix_make: out of memory");
                return nullptr;
        }
        acd::build_matrix(m->h, ncolumns, nrows, nnz, rows, columns, values, permute != 0);
        return m;
}

sparse_matrix_t * sparse_matrix_copy(const sparse_matrix_t * src, int permute)
{
        if (!src)
                return nullptr;
        const acd::HostMatrix & h = src->h;
        return sparse_matrix_make(h.ncols, h.nrows, h.nnz, h.rows.data(), h.cols.data(),
                                  h.vals.data(), permute);
}

int sparse_matrix_free(sparse_matrix_t * m)
{
        if (!m)
                return 0;
        for (auto & v : m->dev)
                for (auto & L : v)
                        if (L.mem)
                                cudaFree(L.mem);
        if (m->scratch)
                cudaFree(m->scratch);
        if (m->stream)
                cudaStreamDestroy(m->stream);
        delete m;
        return 0;
}

size_t sparse_matrix_ncolumns(sparse_matrix_t * m) { return m->h.ncols; }
size_t sparse_matrix_nrows(sparse_matrix_t * m) { return m->h.nrows; }
size_t sparse_matrix_nnz(sparse_matrix_t * m) { return m->h.nnz; }

const uint32_t * sparse_matrix_rows(sparse_matrix_t * m)
{
        acd::ensure_zorder(m->h);
        return m->h.rows.data();
}

const uint32_t * sparse_matrix_columns(sparse_matrix_t * m)
{
        acd::ensure_zorder(m->h);
        return m->h.cols.data();
}

const double * sparse_matrix_values(sparse_matrix_t * m)
{
        acd::ensure_zorder(m->h);
        return m->h.vals.data();
}

static int permute_vec(const acd::Perm & p, double * dest, size_t n, const double * src,
                       int direction)
{
        if (n != p.idx.size())
                return 1;
        const std::vector<uint32_t> & idx = direction >= 0 ? p.idx : p.ridx;
        for (size_t i = 0; i < n; i++)
                dest[i] = src[idx[i]];
        return 0;
}

int sparse_matrix_row_permute(sparse_matrix_t * m, double * dest, size_t n,
                              const double * src, int direction)
{
        return permute_vec(m->h.rperm, dest, n, src, direction);
}

int sparse_matrix_col_permute(sparse_matrix_t * m, double * dest, size_t n,
                              const double * src, int direction)
{
        return permute_vec(m->h.cperm, dest, n, src, direction);
}

int sparse_matrix_multiply(double * OUT_y, size_t ny, const sparse_matrix_t * a,
                           const double * x, size_t nx, int transpose,
                           thread_pool_t * pool)
{
        (void)pool;
        double * y[1] = {OUT_y};
        const double * xs[1] = {x};
        return host_multiply(y, ny, a, xs, nx, transpose != 0, 1);
}

int sparse_matrix_multiply_2(double ** OUT_y, size_t ny, const sparse_matrix_t * a,
                             const double ** x, size_t nx, int transpose,
                             thread_pool_t * pool)
{
        (void)pool;
        return host_multiply(OUT_y, ny, a, x, nx, transpose != 0, 2);
}

sparse_matrix_t * sparse_matrix_read(FILE * stream, int permute)
{
        size_t nrows, ncols, nnz;
        if (!stream || fscanf(stream, " %zu %zu %zu", &nrows, &ncols, &nnz) != 3) {
                acd::set_error(ACDALM_EINVAL, "sparse_matrix_read: bad header");
                return nullptr;
        }
        std::vector<uint32_t> r(nnz), c(nnz);
        std::vector<double> v(nnz);
        for (size_t i = 0; i < nnz; i++)
                if (fscanf(stream, " %u %u %lf", &r[i], &c[i], &v[i]) != 3) {
                        acd::set_error(ACDALM_EINVAL, "sparse_matrix_read: bad triplet %zu", i);
                        return nullptr;
                }
        return sparse_matrix_make(ncols, nrows, nnz, r.data(), c.data(), v.data(), permute);
}

int acdalm_spmv_variant(int variant)
{
        int old = g_variant;
        if (variant >= ACDALM_SPMV_SELL && variant <= ACDALM_SPMV_SELL_FMA)
                g_variant = variant;
        return old;
}

int acdalm_spmv_device(const struct sparse_matrix * ca, int variant, int transpose,
                       const double * x, double * y, void * stream)
{
        sparse_matrix_t * a = const_cast<sparse_matrix_t *>(ca);
        if (variant < 0 || variant > ACDALM_SPMV_SELL_FMA) {
                acd::set_error(ACDALM_EINVAL, "acdalm_spmv_device: variant %d", variant);
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(a->lock);
        return launch<double>(a, variant, transpose != 0, x, nullptr, y, nullptr,
                              (cudaStream_t)stream);
}

int acdalm_spmv_device_f32(const struct sparse_matrix * ca, int variant, int transpose,
                           const float * x, float * y, void * stream)
{
        sparse_matrix_t * a = const_cast<sparse_matrix_t *>(ca);
        if (variant < 0 || variant > ACDALM_SPMV_SELL_FMA) {
                acd::set_error(ACDALM_EINVAL, "acdalm_spmv_device_f32: variant %d", variant);
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(a->lock);
        return launch<float>(a, variant, transpose != 0, x, nullptr, y, nullptr,
                             (cudaStream_t)stream);
}

size_t acdalm_matrix_device_bytes(const struct sparse_matrix * a)
{
        size_t t = 0;
        for (auto & v : a->dev)
                for (auto & L : v)
                        t += L.bytes;
        return t;
}

size_t acdalm_block_bytes(struct sparse_matrix * a, int transpose, size_t * nblocks)
{
        acd::ensure_blocks(a->h);
        const acd::BlockArena & B = transpose ? a->h.block_t : a->h.block;
        *nblocks = B.nblocks;
        return B.bytes.size();
}

int acdalm_block_copy(struct sparse_matrix * a, int transpose, size_t * offsets,
                      void * arena, size_t bytes)
{
        acd::ensure_blocks(a->h);
        const acd::BlockArena & B = transpose ? a->h.block_t : a->h.block;
        if (bytes > B.bytes.size())
                return ACDALM_EINVAL;
        memcpy(offsets, B.offsets.data(), B.nblocks * sizeof(size_t));
        if (bytes)
                memcpy(arena, B.bytes.data(), bytes);
        return 0;
}

int acdalm_csr_copy(struct sparse_matrix * a, int transpose, uint32_t * rows_indices,
                    uint32_t * columns, double * values)
{
        const acd::Csr & c = transpose ? a->h.csr_t : a->h.csr;
        memcpy(rows_indices, c.ptr.data(), (c.nrows + 1) * sizeof(uint32_t));
        if (a->h.nnz) {
                memcpy(columns, c.col.data(), a->h.nnz * sizeof(uint32_t));
                memcpy(values, c.val.data(), a->h.nnz * sizeof(double));
        }
        return 0;
}

int acdalm_sell_copy(struct sparse_matrix * a, int transpose, size_t * nslices,
                     size_t * nelems, int64_t * ptr, int32_t * row0, int32_t * columns,
                     double * values, int32_t * row_of_d)
{
        if (!a || !nslices || !nelems) {
                acd::set_error(ACDALM_EINVAL, "acdalm_sell_copy: null argument");
                return ACDALM_EINVAL;
        }
        acd::PlainSell ps;
        acd::build_plain_sell(a->h, transpose != 0, ps);
        size_t ns = (size_t)ps.s.nslices, ne = (size_t)ps.s.ptr.back();
        if (ptr) {
                if (*nslices < ns || *nelems < ne) {
                        acd::set_error(ACDALM_EINVAL,
                                       "acdalm_sell_copy: %zu slices and %zu elements needed",
                                       ns, ne);
                        return ACDALM_EINVAL;
                }
                memcpy(ptr, ps.s.ptr.data(), (ns + 1) * sizeof(int64_t));
                if (ns)
                        memcpy(row0, ps.s.row0.data(), ns * sizeof(int32_t));
                if (ne) {
                        memcpy(columns, ps.s.col.data(), ne * sizeof(int32_t));
                        memcpy(values, ps.s.val.data(), ne * sizeof(double));
                }
                if (!ps.row_of_d.empty())
                        memcpy(row_of_d, ps.row_of_d.data(), ps.row_of_d.size() * sizeof(int32_t));
        }
        *nslices = ns;
        *nelems = ne;
        return 0;
}

int acdalm_perm_copy(struct sparse_matrix * a, int row, uint32_t * idx, uint32_t * ridx)
{
        const acd::Perm & p = row ? a->h.rperm : a->h.cperm;
        if (!p.idx.empty()) {
                memcpy(idx, p.idx.data(), p.idx.size() * sizeof(uint32_t));
                memcpy(ridx, p.ridx.data(), p.ridx.size() * sizeof(uint32_t));
        }
        return 0;
}

}  // extern "C"


// Internal accessors used by the approx / alm layer.
namespace acd {
void preload_spmv_kernels()
{
        cudaFuncAttributes a;
        cudaFuncGetAttributes(&a, sell_kernel<double, true>);
        cudaFuncGetAttributes(&a, sell_kernel<float, false>);
        cudaFuncGetAttributes(&a, sell2_kernel<double, true>);
        cudaFuncGetAttributes(&a, sell2_kernel<float, false>);
        cudaFuncGetAttributes(&a, sell_kernel<double, false>);
        cudaFuncGetAttributes(&a, sell2_kernel<double, false>);
        cudaFuncGetAttributes(&a, block4_kernel<double>);
        cudaFuncGetAttributes(&a, csr_kernel<double, 4>);
        cudaFuncGetAttributes(&a, csr_kernel<double, 8>);
        cudaFuncGetAttributes(&a, csr_kernel<double, 16>);
        cudaFuncGetAttributes(&a, csr_kernel<double, 32>);
        cudaFuncGetAttributes(&a, csr_kernel<float, 4>);
        cudaFuncGetAttributes(&a, csr_kernel<float, 8>);
        cudaFuncGetAttributes(&a, csr_kernel<float, 16>);
        cudaFuncGetAttributes(&a, csr_kernel<float, 32>);
}
HostMatrix & host_of(sparse_matrix_t * m) { return m->h; }
}
