// Host-side sparse layouts.
//
// Part 1 rebuilds, byte for byte, the layouts the reference keeps for every
// matrix (spmv/spmv.c:27-92): nonzero-count permutations
// (spmv/permutation.c:63-125), CSR of A and A' (spmv/spmv_csr.c:27-80),
// 4-row block arenas (spmv/spmv_block.c:58-149) and the Z-order COO
// (spmv/spmv.swizzle.inc:1-52).  The algorithms are my own (counting sorts
// and radix sorts instead of qsort); the outputs are the reference's.
//
// Part 2 builds the device layout the GPU kernels use: warp-sliced ELL
// ("SELL", one warp per slice) in a device order where rows are sorted by
// length, so a slice's rows have almost no padding.  Within a row, entries
// keep the reference's order (ascending column of the permuted instance),
// so the sequential per-row sums are the reference's sums.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

namespace acd {

struct Csr {
        size_t nrows = 0;
        std::vector<uint32_t> ptr;  // nrows + 1
        std::vector<uint32_t> col;
        std::vector<double> val;
};

struct BlockArena {
        size_t nrows = 0, nblocks = 0;
        std::vector<size_t> offsets;  // byte offset of each block
        std::vector<uint8_t> bytes;   // headers + values + indices
};

struct Perm {
        std::vector<uint32_t> idx;   // new -> old
        std::vector<uint32_t> ridx;  // old -> new
};

struct HostMatrix {
        size_t nrows = 0, ncols = 0, nnz = 0;
        // Triplets after renumbering; Z-ordered lazily (coo_zordered).
        std::vector<uint32_t> rows, cols;
        std::vector<double> vals;
        bool coo_zordered = false;
        Csr csr, csr_t;
        BlockArena block, block_t;  // built lazily (block_ready)
        bool block_ready = false;
        Perm rperm, cperm;
};

// spmv.c:27-92 except the block arenas and the Z-order (built on demand).
void build_matrix(HostMatrix & m, size_t ncols, size_t nrows, size_t nnz,
                  const uint32_t * rows, const uint32_t * cols,
                  const double * vals, bool permute);
void ensure_blocks(HostMatrix & m);
void ensure_zorder(HostMatrix & m);

// Warp-sliced ELL of one operator (A or A') in device order, with a
// per-slice height and lane width.  A slice is 32 lanes wide and holds
// h = 32 / L consecutive rows, each row spread over L lanes (L a power of
// two up to 32, chosen from the slice's longest row).  A slice is either scalar (a
// lane holds V = 1 entry of its row per step) or vector (V = 4 consecutive
// entries per step, so one 16-byte load fetches 4 column indices and one or
// two 16-byte loads their values).  Entry k of the slice's r-th row sits at
// step t = k / (V L), lane q = r L + (k / V) % L, sub-slot k % V, i.e. at
// offset base + 32 V t + V q + k % V.  base = ptr & ~31; the low bits of ptr
// hold log2(L) (bits 0-2) and V = 4 (bit 3).  Within a row, entries keep
// their order (a lane's V entries are consecutive, lanes follow each
// other); padding entries have value 0 and a column of the row.
struct Sell {
        int nrows = 0;                 // rows of the operator
        int nslices = 0;
        std::vector<int64_t> ptr;      // nslices + 1: element offset | log2(L)
        std::vector<int32_t> row0;     // nslices: first row of each slice
        std::vector<int32_t> col;      // ptr[nslices] entries
        std::vector<double> val;
        int max_width = 0;
};

// The device order of a permuted instance and the two SELL operators.
struct DeviceLayout {
        int m = 0, n = 0;
        int64_t nnz = 0;
        // device row d <-> row of the (permuted) instance and the original
        std::vector<int32_t> row_p_of_d, row_d_of_p, row_orig_of_d;
        std::vector<int32_t> col_p_of_d, col_d_of_p, col_orig_of_d;
        std::vector<double> beta;  // nonzeros per device row
        int max_steps = 0;         // the step cap the slices were built with
        Sell a, at;
};

// `pm` is the permuted copy (approx.c:84-88); its CSR orders fix the
// summation order.  Device rows (columns) are the permuted instance's rows
// (columns) sorted by decreasing length, ties by position.
//
// max_steps > 0 spreads the rows of a slice over more lanes (up to 32) until
// the slice takes at most max_steps steps: a team solving one LP on the
// whole GPU waits for its slowest warp every pass, and a warp's time is its
// chain of dependent steps.  0 keeps the width rule alone (teams of one CTA
// or one cluster, which are throughput bound and prefer full lanes).
void build_device_layout(const HostMatrix & pm, DeviceLayout & out, int max_steps);

// The max_steps of layouts for whole-GPU solves (alm_solve, approx_solve,
// mpg_solve): ACDALM_SELL_STEPS, else 8.
int grid_max_steps();

// SELL of a plain matrix (no permutation involved), for the SpMV API:
// device order = rows sorted by length; transpose selects A'.
struct PlainSell {
        std::vector<int32_t> row_of_d;  // device row -> matrix row
        Sell s;
};
void build_plain_sell(const HostMatrix & m, bool transpose, PlainSell & out);

}  // namespace acd
