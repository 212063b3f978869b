// Device builders of the reference's sparse layouts, from COO triplets
// already in device memory: the nonzero-count permutations
// (spmv/permutation.c:63-125) and the CSR of A and A' (spmv/spmv_csr.c:27-80)
// of the optionally permuted matrix -- byte for byte what the host builders
// (layout.cpp, themselves checked against the reference) produce.
//
//  * counts: one atomic increment per triplet into per-row and per-column
//    counters;
//  * permutations: one CTA per window of 256 indices ranks each index by
//    (count, position) -- the stable order the reference's qsort gives
//    within a window;
//  * CSR: the triplets (renumbered) sorted by the 64-bit key (major index,
//    minor index) with a stable least-significant-digit radix sort (8-bit
//    digits, 2,048-key tiles: a per-tile digit histogram, an exclusive scan
//    over (digit, tile), and a scatter that ranks equal digits in the
//    tile's order with warp match masks), then the row pointers by an
//    exclusive scan of the counts.  Keys are unique, so the order is the
//    reference's (row, column) order.
//
// The triplets are checked on the device before any of them indexes an
// array; scratch comes from the stream-ordered allocator on the caller's
// stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/acdalm_ext.h"
#include "common.h"

namespace acd {

namespace {

constexpr int kSortThreads = 256;  // one thread per digit value
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortRounds = 8;     // keys per thread per tile
constexpr int kTile = kSortThreads * kSortRounds;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kWindow = 256;       // permutation.c:59-61
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

static_assert(kSortThreads == kRadix, "the scatter gives each digit one thread");

int grid_for(size_t n, int threads)
{
        size_t b = (n + threads - 1) / threads;
        return (int)std::max<size_t>(1, std::min<size_t>(b, 16384));
}

int bits_for(size_t n)
{
        int b = 1;
        while (b < 32 && ((size_t)1 << b) < n)
                b++;
        return b;
}

// bad[0] = 1 if any triplet's row >= nrows or column >= ncols.
__global__ void check_kernel(const uint32_t * rows, const uint32_t * cols, size_t nnz,
                             size_t nrows, size_t ncols, int * bad)
{
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nnz;
             i += (size_t)gridDim.x * blockDim.x)
                if (rows[i] >= nrows || cols[i] >= ncols)
                        atomicOr(bad, 1);
}

__global__ void count_kernel(const uint32_t * keys, size_t nnz, uint32_t * count)
{
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nnz;
             i += (size_t)gridDim.x * blockDim.x)
                atomicAdd(count + keys[i], 1u);
}

// idx[w + rank(i)] = w + i within each window of kWindow indices, rank by
// (count, position): a stable ascending sort of the window by count.
__global__ void perm_window_kernel(const uint32_t * count, size_t n, uint32_t * idx)
{
        __shared__ uint32_t c[kWindow];
        size_t w = (size_t)blockIdx.x * kWindow;
        int len = (int)std::min<size_t>(kWindow, n - w);
        int i = threadIdx.x;
        if (i < len)
                c[i] = count[w + i];
        __syncthreads();
        if (i < len) {
                uint32_t ci = c[i];
                int rank = 0;
                for (int j = 0; j < len; j++) {
                        uint32_t cj = c[j];
                        rank += (cj < ci) || (cj == ci && j < i);
                }
                idx[w + rank] = (uint32_t)(w + i);
        }
}

__global__ void iota_kernel(uint32_t * idx, size_t n)
{
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
             i += (size_t)gridDim.x * blockDim.x)
                idx[i] = (uint32_t)i;
}

// ridx[idx[p]] = p; cnt_p[p] = count[idx[p]] (the permuted counts), and
// cnt_p[n] = 0 so that an exclusive scan of cnt_p is the row pointer array.
__global__ void invert_kernel(const uint32_t * idx, const uint32_t * count, size_t n,
                              uint32_t * ridx, uint32_t * cnt_p)
{
        for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p <= n;
             p += (size_t)gridDim.x * blockDim.x) {
                if (p == n) {
                        cnt_p[n] = 0;
                        continue;
                }
                uint32_t o = idx[p];
                ridx[o] = (uint32_t)p;
                cnt_p[p] = count[o];
        }
}

// key = (new major << minor_bits) | new minor, payload = triplet index.
__global__ void keys_kernel(const uint32_t * major, const uint32_t * minor,
                            const uint32_t * rmajor, const uint32_t * rminor, size_t nnz,
                            int minor_bits, uint64_t * keys, uint32_t * pos)
{
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nnz;
             i += (size_t)gridDim.x * blockDim.x) {
                uint64_t a = rmajor[major[i]], b = rminor[minor[i]];
                keys[i] = (a << minor_bits) | b;
                pos[i] = (uint32_t)i;
        }
}

// hist[d * ntiles + tile] = keys of the tile whose digit at `shift` is d.
__global__ void __launch_bounds__(kSortThreads) radix_hist_kernel(const uint64_t * keys,
                                                                  size_t nnz, int shift,
                                                                  uint32_t * hist,
                                                                  size_t ntiles)
{
        __shared__ uint32_t h[kRadix];
        int t = threadIdx.x;
        h[t] = 0;
        __syncthreads();
        size_t base = (size_t)blockIdx.x * kTile;
        for (int j = 0; j < kSortRounds; j++) {
                size_t i = base + (size_t)j * kSortThreads + t;
                if (i < nnz)
                        atomicAdd(&h[(keys[i] >> shift) & (kRadix - 1)], 1u);
        }
        __syncthreads();
        hist[(size_t)t * ntiles + blockIdx.x] = h[t];
}

// Stable scatter of one tile: key i goes to offs[d, tile] + (keys of digit d
// before it in the tile).  Round j handles keys base + j * 256 + t, so the
// tile's order is (round, warp, lane); a warp ranks equal digits by match
// masks, and per-digit prefixes over the warps carry the rest.
__global__ void __launch_bounds__(kSortThreads)
radix_scatter_kernel(const uint64_t * keys, const uint32_t * pos, size_t nnz, int shift,
                     const uint32_t * offs, size_t ntiles, uint64_t * keys_out,
                     uint32_t * pos_out)
{
        __shared__ uint32_t next[kRadix];              // where digit d's next key goes
        __shared__ uint32_t wpre[kSortWarps][kRadix];  // per warp: count, then start
        int t = threadIdx.x, lane = t & 31, warp = t >> 5;
        next[t] = offs[(size_t)t * ntiles + blockIdx.x];
        size_t base = (size_t)blockIdx.x * kTile;
        for (int j = 0; j < kSortRounds; j++) {
#pragma unroll
                for (int w = 0; w < kSortWarps; w++)
                        wpre[w][t] = 0;
                __syncthreads();
                size_t i = base + (size_t)j * kSortThreads + t;
                bool valid = i < nnz;
                uint64_t k = valid ? keys[i] : 0;
                uint32_t p = valid ? pos[i] : 0;
                int d = valid ? (int)((k >> shift) & (kRadix - 1)) : kRadix;
                unsigned peers = __match_any_sync(0xffffffffu, d);
                int rank = __popc(peers & ((1u << lane) - 1u));
                if (valid && lane == __ffs(peers) - 1)
                        wpre[warp][d] = __popc(peers);
                __syncthreads();
                {
                        uint32_t run = next[t];
#pragma unroll
                        for (int w = 0; w < kSortWarps; w++) {
                                uint32_t c = wpre[w][t];
                                wpre[w][t] = run;
                                run += c;
                        }
                        next[t] = run;
                }
                __syncthreads();
                if (valid) {
                        uint32_t at = wpre[warp][d] + (uint32_t)rank;
                        keys_out[at] = k;
                        pos_out[at] = p;
                }
                __syncthreads();
        }
}

// In-place exclusive scan of blocks of kScanBlock values; sums[b] = block b's total.
__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(uint32_t * data, size_t n,
                                                                   uint32_t * sums)
{
        __shared__ uint32_t part[kScanThreads];
        size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanItems;
        uint32_t v[kScanItems];
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
                v[k] = (base + k < n) ? data[base + k] : 0u;
                uint32_t c = v[k];
                v[k] = s;
                s += c;
        }
        part[threadIdx.x] = s;
        __syncthreads();
        // Hillis-Steele over the threads' totals
        for (int off = 1; off < kScanThreads; off <<= 1) {
                uint32_t add = (threadIdx.x >= (unsigned)off) ? part[threadIdx.x - off] : 0u;
                __syncthreads();
                part[threadIdx.x] += add;
                __syncthreads();
        }
        uint32_t before = (threadIdx.x > 0) ? part[threadIdx.x - 1] : 0u;
#pragma unroll
        for (int k = 0; k < kScanItems; k++)
                if (base + k < n)
                        data[base + k] = v[k] + before;
        if (threadIdx.x == kScanThreads - 1)
                sums[blockIdx.x] = part[kScanThreads - 1];
}

// Exclusive scan of the block totals in one CTA, chunk by chunk.
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(uint32_t * sums, size_t n)
{
        __shared__ uint32_t part[kScanThreads];
        __shared__ uint32_t carry;
        if (threadIdx.x == 0)
                carry = 0;
        __syncthreads();
        for (size_t c0 = 0; c0 < n; c0 += kScanThreads) {
                size_t i = c0 + threadIdx.x;
                uint32_t v = (i < n) ? sums[i] : 0u;
                part[threadIdx.x] = v;
                __syncthreads();
                for (int off = 1; off < kScanThreads; off <<= 1) {
                        uint32_t add = (threadIdx.x >= (unsigned)off) ? part[threadIdx.x - off]
                                                                      : 0u;
                        __syncthreads();
                        part[threadIdx.x] += add;
                        __syncthreads();
                }
                uint32_t incl = part[threadIdx.x];
                uint32_t base = carry;
                if (i < n)
                        sums[i] = base + incl - v;
                __syncthreads();
                if (threadIdx.x == kScanThreads - 1)
                        carry = base + incl;
                __syncthreads();
        }
}

__global__ void add_sums_kernel(uint32_t * data, size_t n, const uint32_t * sums)
{
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
             i += (size_t)gridDim.x * blockDim.x)
                data[i] += sums[i / kScanBlock];
}

// col[j] = minor of sorted key j, val[j] = vals[payload j].
__global__ void csr_out_kernel(const uint64_t * keys, const uint32_t * pos, size_t nnz,
                               int minor_bits, const double * vals, uint32_t * col,
                               double * val)
{
        uint64_t mask = (minor_bits >= 64) ? ~0ull : ((1ull << minor_bits) - 1ull);
        for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < nnz;
             j += (size_t)gridDim.x * blockDim.x) {
                col[j] = (uint32_t)(keys[j] & mask);
                val[j] = vals[pos[j]];
        }
}

struct Scratch {
        char * base = nullptr;
        cudaStream_t s = nullptr;
        ~Scratch()
        {
                if (base)
                        cudaFreeAsync(base, s);
        }
};

// Exclusive scan of data[0..n) in place, with `sums` room for the block totals.
int exclusive_scan(uint32_t * data, size_t n, uint32_t * sums, cudaStream_t s)
{
        if (n == 0)
                return 0;
        size_t nb = (n + kScanBlock - 1) / kScanBlock;
        scan_blocks_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(data, n, sums);
        scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, nb);
        add_sums_kernel<<<grid_for(n, 256), 256, 0, s>>>(data, n, sums);
        count_launch(3);
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        return 0;
}

// Stable sort of (keys, pos) by the low `bits` bits of the keys; the result
// ends in keys / pos (the *2 arrays are the other buffer).
int radix_sort(uint64_t *& keys, uint32_t *& pos, uint64_t *& keys2, uint32_t *& pos2,
               size_t nnz, int bits, uint32_t * hist, uint32_t * sums, cudaStream_t s)
{
        if (nnz == 0)
                return 0;
        size_t ntiles = (nnz + kTile - 1) / kTile;
        for (int shift = 0; shift < bits; shift += kRadixBits) {
                radix_hist_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(keys, nnz, shift, hist,
                                                                          ntiles);
                count_launch();
                int r = exclusive_scan(hist, (size_t)kRadix * ntiles, sums, s);
                if (r)
                        return r;
                radix_scatter_kernel<<<(unsigned)ntiles, kSortThreads, 0, s>>>(
                        keys, pos, nnz, shift, hist, ntiles, keys2, pos2);
                count_launch();
                ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
                std::swap(keys, keys2);
                std::swap(pos, pos2);
        }
        return 0;
}

template <class T>
T * carve(char *& p, size_t count)
{
        T * r = reinterpret_cast<T *>(p);
        p += (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
        return r;
}

}  // namespace

}  // namespace acd

extern "C" int acdalm_layout_device(size_t nrows, size_t ncols, size_t nnz,
                                    const uint32_t * rows, const uint32_t * cols,
                                    const double * values, int permute,
                                    uint32_t * row_idx, uint32_t * col_idx, uint32_t * ptr,
                                    uint32_t * columns, double * vals, uint32_t * ptr_t,
                                    uint32_t * columns_t, double * vals_t, void * stream)
{
        using namespace acd;
        if (nrows >= (1ull << 32) || ncols >= (1ull << 32) || nnz >= (1ull << 32)
            || (nnz && (!rows || !cols || !values || !columns || !vals || !columns_t || !vals_t))
            || (nrows && !row_idx) || (ncols && !col_idx) || !ptr || !ptr_t) {
                set_error(ACDALM_EINVAL, "acdalm_layout_device: sizes or NULL arrays");
                return ACDALM_EINVAL;
        }
        if (!device_ready())
                return ACDALM_ENODEV;
        NvtxRange range("acdalm layout build");
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        size_t ntiles = (nnz + kTile - 1) / kTile;
        size_t scanned = std::max(std::max(nrows, ncols) + 1, (size_t)kRadix * ntiles);
        size_t nsums = (scanned + kScanBlock - 1) / kScanBlock + 1;
        size_t bytes = 0;
        auto need = [&](size_t count, size_t size) {
                bytes += (std::max<size_t>(count, 1) * size + 255) & ~size_t(255);
        };
        need(1, sizeof(int));                               // bad
        need(nrows + 1, 4); need(ncols + 1, 4);              // counts
        need(nrows, 4); need(ncols, 4);                      // ridx
        need(nrows + 1, 4); need(ncols + 1, 4);              // permuted counts
        need(nnz, 8); need(nnz, 8); need(nnz, 4); need(nnz, 4);
        need((size_t)kRadix * ntiles, 4);
        need(nsums, 4);
        Scratch sc;
        sc.s = s;
        {
                void * p = nullptr;
                cudaError_t e = cudaMallocAsync(&p, bytes, s);
                if (e != cudaSuccess) {
                        set_error(ACDALM_ENOMEM, "acdalm_layout_device: %zu bytes of scratch: %s",
                                  bytes, cudaGetErrorString(e));
                        return ACDALM_ENOMEM;
                }
                sc.base = static_cast<char *>(p);
        }
        char * p = sc.base;
        int * bad = carve<int>(p, 1);
        uint32_t * rcount = carve<uint32_t>(p, nrows + 1);
        uint32_t * ccount = carve<uint32_t>(p, ncols + 1);
        uint32_t * rridx = carve<uint32_t>(p, nrows);
        uint32_t * cridx = carve<uint32_t>(p, ncols);
        uint32_t * rcnt_p = carve<uint32_t>(p, nrows + 1);
        uint32_t * ccnt_p = carve<uint32_t>(p, ncols + 1);
        uint64_t * keys = carve<uint64_t>(p, nnz);
        uint64_t * keys2 = carve<uint64_t>(p, nnz);
        uint32_t * pos = carve<uint32_t>(p, nnz);
        uint32_t * pos2 = carve<uint32_t>(p, nnz);
        uint32_t * hist = carve<uint32_t>(p, (size_t)kRadix * ntiles);
        uint32_t * sums = carve<uint32_t>(p, nsums);

        // the triplets index the count arrays: check them first
        ACD_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s), ACDALM_ECUDA);
        if (nnz) {
                check_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(rows, cols, nnz, nrows, ncols, bad);
                count_launch();
        }
        int hbad = 0;
        ACD_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s),
                     ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(s), ACDALM_ECUDA);
        if (hbad) {
                set_error(ACDALM_EINVAL, "acdalm_layout_device: a triplet is out of range");
                return ACDALM_EINVAL;
        }
        ACD_CUDA_TRY(cudaMemsetAsync(rcount, 0, (nrows + 1) * 4, s), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemsetAsync(ccount, 0, (ncols + 1) * 4, s), ACDALM_ECUDA);
        if (nnz) {
                count_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(rows, nnz, rcount);
                count_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(cols, nnz, ccount);
                count_launch(2);
        }
        // permutations (permutation.c:63-125) or the identity
        if (permute) {
                if (nrows)
                        perm_window_kernel<<<(unsigned)((nrows + kWindow - 1) / kWindow), kWindow, 0,
                                             s>>>(rcount, nrows, row_idx);
                if (ncols)
                        perm_window_kernel<<<(unsigned)((ncols + kWindow - 1) / kWindow), kWindow, 0,
                                             s>>>(ccount, ncols, col_idx);
        } else {
                if (nrows)
                        iota_kernel<<<grid_for(nrows, 256), 256, 0, s>>>(row_idx, nrows);
                if (ncols)
                        iota_kernel<<<grid_for(ncols, 256), 256, 0, s>>>(col_idx, ncols);
        }
        invert_kernel<<<grid_for(nrows + 1, 256), 256, 0, s>>>(row_idx, rcount, nrows, rridx,
                                                               rcnt_p);
        invert_kernel<<<grid_for(ncols + 1, 256), 256, 0, s>>>(col_idx, ccount, ncols, cridx,
                                                               ccnt_p);
        count_launch(4);
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        // row pointers: exclusive scans of the permuted counts
        int r;
        if ((r = exclusive_scan(rcnt_p, nrows + 1, sums, s)) ||
            (r = exclusive_scan(ccnt_p, ncols + 1, sums, s)))
                return r;
        ACD_CUDA_TRY(cudaMemcpyAsync(ptr, rcnt_p, (nrows + 1) * 4, cudaMemcpyDeviceToDevice, s),
                     ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemcpyAsync(ptr_t, ccnt_p, (ncols + 1) * 4, cudaMemcpyDeviceToDevice,
                                     s), ACDALM_ECUDA);
        // CSR of A by (row, column), of A' by (column, row)
        int rbits = bits_for(nrows), cbits = bits_for(ncols);
        for (int t = 0; t < 2 && nnz; t++) {
                const uint32_t * major = t ? cols : rows;
                const uint32_t * minor = t ? rows : cols;
                const uint32_t * rmaj = t ? cridx : rridx;
                const uint32_t * rmin = t ? rridx : cridx;
                int minor_bits = t ? rbits : cbits;
                keys_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(major, minor, rmaj, rmin, nnz,
                                                              minor_bits, keys, pos);
                count_launch();
                uint64_t * k1 = keys, * k2 = keys2;
                uint32_t * p1 = pos, * p2 = pos2;
                if ((r = radix_sort(k1, p1, k2, p2, nnz, rbits + cbits, hist, sums, s)))
                        return r;
                csr_out_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(
                        k1, p1, nnz, minor_bits, values, t ? columns_t : columns, t ? vals_t : vals);
                count_launch();
                ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        }
        ACD_CUDA_TRY(cudaStreamSynchronize(s), ACDALM_ECUDA);
        return 0;
}
