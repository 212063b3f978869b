// Host-side sparse layouts; see layout.h.
#include "layout.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>

namespace acd {

namespace {

constexpr size_t kBlockRows = 4;       // spmv_block.h:3-5
constexpr size_t kBlockRing = 16;      // spmv_block.c:143-145
constexpr size_t kBlockHeader = 32;    // sizeof(struct matrix_subblock)
constexpr size_t kSortWindow = 256;    // permutation.c:59-61
constexpr int kSlice = 32;             // rows per SELL slice (one warp)
constexpr int kVec = 4;                // entries per lane per step, vector slices
constexpr int64_t kVecFlag = 8;        // slice pointer bit: vector slice

// permutation.c:63-125: nonzeros per index; each window of 256 sorted by
// (count, original index).  A stable counting of the window by count gives
// exactly that order.
void build_perm(Perm & p, const uint32_t * keys, size_t nnz, size_t n)
{
        std::vector<uint32_t> count(n, 0);
        for (size_t i = 0; i < nnz; i++)
                count[keys[i]]++;
        p.idx.resize(n);
        p.ridx.resize(n);
        std::iota(p.idx.begin(), p.idx.end(), 0u);
        for (size_t w = 0; w < n; w += kSortWindow) {
                size_t e = std::min(n, w + kSortWindow);
                std::stable_sort(p.idx.begin() + w, p.idx.begin() + e,
                                 [&](uint32_t a, uint32_t b) {
                                         return count[a] < count[b];
                                 });
        }
        for (size_t i = 0; i < n; i++)
                p.ridx[p.idx[i]] = (uint32_t)i;
}

void identity_perm(Perm & p, size_t n)
{
        p.idx.resize(n);
        p.ridx.resize(n);
        std::iota(p.idx.begin(), p.idx.end(), 0u);
        std::iota(p.ridx.begin(), p.ridx.end(), 0u);
}

// spmv_csr.c:27-80: entries ordered by (row, column); ptr[r+1] = end of row
// r.  Keys are unique, so a counting sort by row followed by sorting each
// row by column reproduces the reference's qsort order exactly.
void build_csr(Csr & c, const uint32_t * major, const uint32_t * minor,
               const double * vals, size_t nnz, size_t n)
{
        c.nrows = n;
        c.ptr.assign(n + 1, 0);
        for (size_t i = 0; i < nnz; i++)
                c.ptr[major[i] + 1]++;
        for (size_t r = 0; r < n; r++)
                c.ptr[r + 1] += c.ptr[r];
        c.col.resize(nnz);
        c.val.resize(nnz);
        std::vector<uint32_t> fill(c.ptr.begin(), c.ptr.end() - 1);
        for (size_t i = 0; i < nnz; i++) {
                uint32_t at = fill[major[i]]++;
                c.col[at] = minor[i];
                c.val[at] = vals[i];
        }
        std::vector<std::pair<uint32_t, double>> tmp;
        for (size_t r = 0; r < n; r++) {
                uint32_t b = c.ptr[r], e = c.ptr[r + 1];
                bool sorted = true;
                for (uint32_t j = b + 1; j < e && sorted; j++)
                        sorted = c.col[j - 1] < c.col[j];
                if (sorted)
                        continue;
                tmp.clear();
                for (uint32_t j = b; j < e; j++)
                        tmp.emplace_back(c.col[j], c.val[j]);
                std::sort(tmp.begin(), tmp.end(),
                          [](const auto & x, const auto & y) {
                                  return x.first < y.first;
                          });
                for (uint32_t j = b; j < e; j++) {
                        c.col[j] = tmp[j - b].first;
                        c.val[j] = tmp[j - b].second;
                }
        }
}

size_t block_bytes(size_t width)
{
        size_t b = kBlockHeader
                + (sizeof(double) + sizeof(uint32_t)) * kBlockRows * width;
        return (b + 63) & ~size_t(63);
}

// spmv_block.c:58-149; see make_single_block for the padding rule: scanning
// a block's slots backwards, a slot holding 0.0 takes the next column of a
// 16-entry ring that records the columns of the non-zero slots seen so far.
void build_block(BlockArena & b, const Csr & c)
{
        size_t nrows = c.nrows;
        size_t nblocks = (nrows + kBlockRows - 1) / kBlockRows;
        b.nrows = nrows;
        b.nblocks = nblocks;
        b.offsets.resize(nblocks);
        std::vector<uint32_t> width(nblocks, 0);
        size_t total = 0;
        for (size_t k = 0; k < nblocks; k++) {
                size_t start = k * kBlockRows;
                size_t end = std::min(nrows, start + kBlockRows);
                uint32_t w = 0;
                for (size_t r = start; r < end; r++)
                        w = std::max(w, c.ptr[r + 1] - c.ptr[r]);
                width[k] = w;
                b.offsets[k] = total;
                total += block_bytes(w);
        }
        b.bytes.assign(total, 0);
        for (size_t k = 0; k < nblocks; k++) {
                uint8_t * base = b.bytes.data() + b.offsets[k];
                size_t start = k * kBlockRows;
                size_t nr = std::min(kBlockRows, nrows - start);
                size_t w = width[k], slots = kBlockRows * w;
                double * vals = reinterpret_cast<double *>(base + kBlockHeader);
                uint32_t * cols = reinterpret_cast<uint32_t *>(vals + slots);
                for (size_t r = 0; r < nr; r++) {
                        size_t s = r;
                        for (uint32_t j = c.ptr[start + r];
                             j < c.ptr[start + r + 1]; j++, s += kBlockRows) {
                                cols[s] = c.col[j];
                                vals[s] = c.val[j];
                        }
                }
                uint32_t ring[kBlockRing] = {0};
                size_t rd = 0, wr = 0;
                for (size_t s = slots; s-- > 0;) {
                        if (vals[s] == 0) {
                                cols[s] = ring[rd];
                                rd = (rd + 1) % kBlockRing;
                        } else {
                                ring[wr] = cols[s];
                                wr = (wr + 1) % kBlockRing;
                        }
                }
                uint32_t hdr[3] = {(uint32_t)w, (uint32_t)start, (uint32_t)nr};
                std::memcpy(base, hdr, sizeof(hdr));
        }
}

// Spread the 32 bits of v to the even bit positions of a 64-bit word.
inline uint64_t spread_bits(uint32_t v)
{
        uint64_t x = v;
        x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
        x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
        x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
        x = (x | (x << 2)) & 0x3333333333333333ull;
        x = (x | (x << 1)) & 0x5555555555555555ull;
        return x;
}

}  // namespace

void build_matrix(HostMatrix & m, size_t ncols, size_t nrows, size_t nnz,
                  const uint32_t * rows, const uint32_t * cols,
                  const double * vals, bool permute)
{
        m.nrows = nrows;
        m.ncols = ncols;
        m.nnz = nnz;
        m.rows.assign(rows, rows + nnz);
        m.cols.assign(cols, cols + nnz);
        m.vals.assign(vals, vals + nnz);
        m.coo_zordered = false;
        m.block_ready = false;
        if (permute) {
                build_perm(m.rperm, m.rows.data(), nnz, nrows);
                build_perm(m.cperm, m.cols.data(), nnz, ncols);
                for (size_t i = 0; i < nnz; i++) {
                        m.rows[i] = m.rperm.ridx[m.rows[i]];
                        m.cols[i] = m.cperm.ridx[m.cols[i]];
                }
        } else {
                identity_perm(m.rperm, nrows);
                identity_perm(m.cperm, ncols);
        }
        build_csr(m.csr, m.rows.data(), m.cols.data(), m.vals.data(), nnz,
                  nrows);
        build_csr(m.csr_t, m.cols.data(), m.rows.data(), m.vals.data(), nnz,
                  ncols);
}

void ensure_blocks(HostMatrix & m)
{
        if (m.block_ready)
                return;
        build_block(m.block, m.csr);
        build_block(m.block_t, m.csr_t);
        m.block_ready = true;
}

// spmv.swizzle.inc:14-52: the triplets sorted by Morton key (column bits
// even, row bits odd).  Keys are unique; an LSD radix sort on 16-bit digits
// gives the same order as the reference's qsort.
void ensure_zorder(HostMatrix & m)
{
        if (m.coo_zordered)
                return;
        size_t nnz = m.nnz;
        std::vector<uint64_t> key(nnz), key2(nnz);
        std::vector<uint32_t> pos(nnz), pos2(nnz);
        for (size_t i = 0; i < nnz; i++) {
                key[i] = spread_bits(m.cols[i]) | (spread_bits(m.rows[i]) << 1);
                pos[i] = (uint32_t)i;
        }
        std::vector<size_t> hist(1u << 16);
        for (int pass = 0; pass < 4; pass++) {
                int shift = 16 * pass;
                std::fill(hist.begin(), hist.end(), 0);
                for (size_t i = 0; i < nnz; i++)
                        hist[(key[i] >> shift) & 0xffff]++;
                size_t run = 0;
                for (auto & h : hist) {
                        size_t c = h;
                        h = run;
                        run += c;
                }
                for (size_t i = 0; i < nnz; i++) {
                        size_t at = hist[(key[i] >> shift) & 0xffff]++;
                        key2[at] = key[i];
                        pos2[at] = pos[i];
                }
                key.swap(key2);
                pos.swap(pos2);
        }
        std::vector<uint32_t> r(nnz), c(nnz);
        std::vector<double> v(nnz);
        for (size_t i = 0; i < nnz; i++) {
                r[i] = m.rows[pos[i]];
                c[i] = m.cols[pos[i]];
                v[i] = m.vals[pos[i]];
        }
        m.rows.swap(r);
        m.cols.swap(c);
        m.vals.swap(v);
        m.coo_zordered = true;
}

namespace {

// Positions 0..n-1 sorted by decreasing length, ties by position (a stable
// counting sort on the length).
std::vector<int32_t> order_by_length(const std::vector<uint32_t> & ptr)
{
        size_t n = ptr.size() - 1;
        uint32_t maxlen = 0;
        for (size_t i = 0; i < n; i++)
                maxlen = std::max(maxlen, ptr[i + 1] - ptr[i]);
        std::vector<size_t> start(maxlen + 2, 0);
        for (size_t i = 0; i < n; i++)
                start[maxlen - (ptr[i + 1] - ptr[i]) + 1]++;
        for (size_t k = 1; k < start.size(); k++)
                start[k] += start[k - 1];
        std::vector<int32_t> order(n);
        for (size_t i = 0; i < n; i++)
                order[start[maxlen - (ptr[i + 1] - ptr[i])]++] = (int32_t)i;
        return order;
}

// Lanes per row for a slice whose longest row has `len` entries.
int lanes_for(uint32_t len)
{
        if (len <= 16)
                return 1;
        if (len <= 64)
                return 4;
        if (len <= 256)
                return 16;
        return 32;
}

int log2i(int v)
{
        int r = 0;
        while ((1 << r) < v)
                r++;
        return r;
}

// How slices pick between scalar lanes (one entry per lane per step) and
// vector lanes (4 consecutive entries per lane per step, 16-byte loads):
// ACDALM_SELL_VEC=0 never vectorises, 1 always, unset / "auto" vectorises a
// slice when its rows' capacity grows by at most 1/8 over the scalar
// form's (rounding a row up to a multiple of 4L adds padding, and every
// padding entry still costs a gather).
int vector_mode()
{
        const char * e = getenv("ACDALM_SELL_VEC");
        if (e && e[0] == '0')
                return 0;
        if (e && e[0] == '1')
                return 1;
        return 2;
}

// One SELL operator: device row d is CSR row src_of_d[d] (rows already in
// decreasing length); its entries keep their CSR order, columns mapped
// through col_map (identity if empty).
void build_sell(Sell & s, const Csr & c, const std::vector<int32_t> & src_of_d,
                const std::vector<int32_t> & col_map, int max_steps)
{
        int n = (int)src_of_d.size();
        int mode = vector_mode();
        s.nrows = n;
        s.ptr.clear();
        s.row0.clear();
        s.max_width = 0;
        auto len_of = [&](int d) { return c.ptr[src_of_d[d] + 1] - c.ptr[src_of_d[d]]; };
        auto cdiv = [](uint32_t a, uint32_t b) { return (a + b - 1) / b; };
        struct Shape {
                int L, vec;
        };
        std::vector<Shape> shape;
        int64_t off = 0;
        for (int d = 0; d < n;) {
                uint32_t first = len_of(d);
                int L1 = lanes_for(first), L4 = lanes_for(cdiv(first, kVec));
                if (max_steps > 0) {
                        // more lanes per row until the slice takes at most
                        // max_steps steps (rows are in decreasing length, so
                        // the first row is the slice's longest)
                        while (L1 < kSlice && cdiv(first, L1) > (uint32_t)max_steps)
                                L1 *= 2;
                        while (L4 < kSlice && cdiv(first, kVec * L4) > (uint32_t)max_steps)
                                L4 *= 2;
                }
                uint32_t cap1 = cdiv(first, L1) * L1, cap4 = cdiv(first, kVec * L4) * kVec * L4;
                bool vec = mode == 1 || (mode == 2 && 8 * (uint64_t)cap4 <= 9 * (uint64_t)cap1);
                int L = vec ? L4 : L1, V = vec ? kVec : 1;
                int h = kSlice / L;
                uint32_t w = 0;
                for (int r = d; r < std::min(n, d + h); r++)
                        w = std::max(w, len_of(r));
                s.max_width = std::max(s.max_width, (int)w);
                int64_t steps = cdiv(w, (uint32_t)(V * L));
                s.ptr.push_back(off | log2i(L) | (vec ? kVecFlag : 0));
                s.row0.push_back(d);
                shape.push_back({L, V});
                off += steps * kSlice * V;
                d += h;
        }
        s.nslices = (int)s.row0.size();
        s.ptr.push_back(off);
        s.col.assign(off, 0);
        s.val.assign(off, 0.0);
        auto map = [&](uint32_t cc) {
                return col_map.empty() ? (int32_t)cc : col_map[cc];
        };
        // entry k of row r of a slice: step k / (V L), lane r L + (k / V) % L,
        // sub-slot k % V
        auto at = [](int64_t base, Shape sh, int r, uint32_t k) {
                int64_t step = k / (sh.vec * sh.L);
                int q = r * sh.L + (int)((k / sh.vec) % sh.L);
                return base + step * (kSlice * sh.vec) + q * sh.vec + k % sh.vec;
        };
        for (int sl = 0; sl < s.nslices; sl++) {
                int64_t base = s.ptr[sl] & ~int64_t(kSlice - 1);
                Shape sh = shape[sl];
                int h = kSlice / sh.L;
                int64_t end = s.ptr[sl + 1] & ~int64_t(kSlice - 1);
                uint32_t slots = (uint32_t)((end - base) / kSlice) * sh.L;
                int d0 = s.row0[sl];
                int32_t slice_pad = 0;
                for (int r = 0; r < h && d0 + r < n; r++) {
                        int src = src_of_d[d0 + r];
                        if (c.ptr[src + 1] > c.ptr[src]) {
                                slice_pad = map(c.col[c.ptr[src]]);
                                break;
                        }
                }
                for (int r = 0; r < h; r++) {
                        int d = d0 + r;
                        int32_t pad = slice_pad;
                        uint32_t k = 0;
                        if (d < n) {
                                int src = src_of_d[d];
                                for (uint32_t j = c.ptr[src]; j < c.ptr[src + 1]; j++, k++) {
                                        int64_t o = at(base, sh, r, k);
                                        s.col[o] = map(c.col[j]);
                                        s.val[o] = c.val[j];
                                        pad = s.col[o];
                                }
                        }
                        // padding: value 0, a column of this row (or slice),
                        // so the gather stays in cache and in bounds
                        for (; k < slots; k++)
                                s.col[at(base, sh, r, k)] = pad;
                }
        }
}

}  // namespace

int grid_max_steps()
{
        const char * e = getenv("ACDALM_SELL_STEPS");
        return e ? atoi(e) : 8;
}

void build_device_layout(const HostMatrix & pm, DeviceLayout & out, int max_steps)
{
        int m = (int)pm.nrows, n = (int)pm.ncols;
        out.m = m;
        out.n = n;
        out.nnz = (int64_t)pm.nnz;
        out.row_p_of_d = order_by_length(pm.csr.ptr);
        out.col_p_of_d = order_by_length(pm.csr_t.ptr);
        out.row_d_of_p.assign(m, 0);
        out.col_d_of_p.assign(n, 0);
        out.row_orig_of_d.assign(m, 0);
        out.col_orig_of_d.assign(n, 0);
        out.beta.assign(m, 0.0);
        for (int d = 0; d < m; d++) {
                int p = out.row_p_of_d[d];
                out.row_d_of_p[p] = d;
                out.row_orig_of_d[d] = (int32_t)pm.rperm.idx[p];
                out.beta[d] = (double)(pm.csr.ptr[p + 1] - pm.csr.ptr[p]);
        }
        for (int d = 0; d < n; d++) {
                int p = out.col_p_of_d[d];
                out.col_d_of_p[p] = d;
                out.col_orig_of_d[d] = (int32_t)pm.cperm.idx[p];
        }
        out.max_steps = max_steps;
        build_sell(out.a, pm.csr, out.row_p_of_d, out.col_d_of_p, max_steps);
        build_sell(out.at, pm.csr_t, out.col_p_of_d, out.row_d_of_p, max_steps);
}

void build_plain_sell(const HostMatrix & m, bool transpose, PlainSell & out)
{
        const Csr & c = transpose ? m.csr_t : m.csr;
        out.row_of_d = order_by_length(c.ptr);
        build_sell(out.s, c, out.row_of_d, {}, 0);
}

}  // namespace acd
