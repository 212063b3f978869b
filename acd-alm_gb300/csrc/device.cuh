// Device primitives shared by the kernels: teams of threads that run one
// solve together, deterministic reductions, bounded waits, SELL row loops.
//
// A "team" is the set of threads that cooperate on one LP.  Every thread of
// a team executes the same control flow (the solver's scalars are computed
// redundantly from identical reduction results), data-parallel phases split
// rows over the team's warps, and team.reduce() is both the reduction and
// the barrier between phases.
//
//   GridTeam    - every CTA of a cooperative launch (one large LP).  Each
//                 CTA publishes its partials in its own line, every word
//                 tagged with the reduction's epoch; every CTA polls all
//                 lines until the tags match and sums them itself in CTA
//                 order, so every CTA reads the same bits.
//   BlockTeam   - one CTA (one small LP of a batch); __syncthreads based.
//   ClusterTeam - the CTAs of one thread-block cluster (a large served LP);
//                 partials read through distributed shared memory, hardware
//                 cluster barriers.
//
// No wait is unbounded: a CTA that waits more than kWaitLimitNs for the
// others records ACDALM_ETIMEOUT in the team's status word and every thread
// returns; nothing traps.
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

namespace acd {

constexpr int kWarp = 32;
constexpr int kRedMax = 8;                           // values per reduction
constexpr unsigned long long kWaitLimitNs = 20ull * 1000000000ull;
constexpr int kStatusTimeout = -2;                   // ACDALM_ETIMEOUT
constexpr int kStatusNonFinite = -5;                 // ACDALM_ENONFINITE
constexpr int kStatusTimeLimit = -7;                 // ACDALM_ETIMELIMIT
constexpr int kStatusInternal = -4;                  // ACDALM_EINVAL: an internal
                                                     // invariant did not hold

enum RedOp { RED_SUM = 0, RED_MAX = 1, RED_MIN = 2 };

// A float-float number hi + lo (|lo| <= ulp(hi) / 2 after normalisation):
// the FP32 inner solve accumulates its reduction partials in this form on
// the FP32 pipe, which is many times wider than the FP64 pipe of this GPU.
// A product of two floats is carried exactly (Dekker's two-product via one
// fused multiply-add), sums use Knuth's two-sum, so a partial over a few
// hundred terms keeps about 44 bits.
struct DF {
        float hi, lo;
};

// a + b exactly as s + e (Knuth's two-sum; no multiplications, so nothing
// is contracted).
__device__ __forceinline__ void two_sum(float a, float b, float & s, float & e)
{
        s = a + b;
        float bb = s - a;
        e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ DF df_add(DF a, DF b)
{
        float s, e;
        two_sum(a.hi, b.hi, s, e);
        e += a.lo + b.lo;
        float h = s + e;
        return {h, e - (h - s)};
}

// Partial accumulators: double for the FP64 solve, DF for the FP32 one.
__device__ __forceinline__ void acc_add(double & a, double x) { a += x; }
__device__ __forceinline__ void acc_prod(double & a, double x, double y) { a += x * y; }
__device__ __forceinline__ void acc_max(double & a, double x) { a = (x > a) ? x : a; }

__device__ __forceinline__ void acc_add(DF & a, float x)
{
        float s, e;
        two_sum(a.hi, x, s, e);
        a.hi = s;
        a.lo += e;
}

// a += x for a double term of the FP32 solve (the rare terms that involve
// the FP64 point): x split into two floats.
__device__ __forceinline__ void acc_add(DF & a, double x)
{
        float h = (float)x;
        acc_add(a, h);
        a.lo += (float)(x - (double)h);
}

__device__ __forceinline__ void acc_prod(DF & a, float x, float y)
{
        float p = __fmul_rn(x, y);
        float pe = fmaf(x, y, -p);  // exact: x y = p + pe
        acc_add(a, p);
        a.lo += pe;
}

__device__ __forceinline__ void acc_max(DF & a, float x)
{
        if (x > a.hi)
                a = {x, 0.f};
}

__device__ __forceinline__ double red_identity(int op)
{
        return op == RED_SUM ? 0.0 : (op == RED_MAX ? -HUGE_VAL : HUGE_VAL);
}

__device__ __forceinline__ double red_combine(int op, double a, double b)
{
        if (op == RED_SUM)
                return a + b;
        if (op == RED_MAX)
                return (b > a) ? b : a;
        return (b < a) ? b : a;
}

__device__ __forceinline__ DF red_combine(int op, DF a, DF b)
{
        if (op == RED_SUM)
                return df_add(a, b);
        if (op == RED_MAX)
                return (b.hi > a.hi) ? b : a;
        return (b.hi < a.hi) ? b : a;
}

template <class P>
__device__ __forceinline__ P red_identity_as(int op);
template <>
__device__ __forceinline__ double red_identity_as<double>(int op) { return red_identity(op); }
template <>
__device__ __forceinline__ DF red_identity_as<DF>(int op)
{
        float v = op == RED_SUM ? 0.f : (op == RED_MAX ? -HUGE_VALF : HUGE_VALF);
        return {v, 0.f};
}

__device__ __forceinline__ double shfl_down(double v, int o)
{
        return __shfl_down_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ DF shfl_down(DF v, int o)
{
        return {__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(DF v) { return (double)v.hi + (double)v.lo; }

__device__ __forceinline__ unsigned long long global_ns()
{
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned * p)
{
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p)
                     : "memory");
        return v;
}

__device__ __forceinline__ int ld_relaxed_int(const int * p)
{
        int v;
        asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p)
                     : "memory");
        return v;
}

__device__ __forceinline__ int ld_acquire_int(const int * p)
{
        int v;
        asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p)
                     : "memory");
        return v;
}

// Lane 0 of each warp ends with the warp's combination (fixed tree order).
template <class P>
__device__ __forceinline__ P warp_reduce(P v, int op)
{
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
                v = red_combine(op, v, shfl_down(v, o));
        return v;
}

__device__ __forceinline__ double shfl_xor(double v, int o)
{
        return __shfl_xor_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ DF shfl_xor(DF v, int o)
{
        return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// Warp reduction of KP = 1, 2, 4 or 8 values at once (a transposing
// butterfly): at offsets 16, 8, ... each lane keeps half of its slots --
// the upper half if its lane bit is set -- and adds its partner's copy of
// them, so each level costs KP/2 additions instead of KP; after log2 KP
// levels every lane holds one slot, and a plain tree over the remaining
// 32/KP lanes finishes it.  Slot k's total ends in lane k * (32/KP).  For
// KP = 8 that is 9 additions per lane where 8 separate trees take 40: on
// this GPU's narrow FP64 pipe, most of the cost of a block reduction.  The
// order of the additions is fixed, so the result is deterministic.
template <int KP, class P>
__device__ __forceinline__ P warp_reduce_many(P (&v)[KP], int (&op)[KP], int lane)
{
#pragma unroll
        for (int h = KP / 2, off = 16; h >= 1; h /= 2, off /= 2) {
                bool hi = (lane & off) != 0;
#pragma unroll
                for (int j = 0; j < h; j++) {
                        P keep = hi ? v[h + j] : v[j];
                        P give = hi ? v[j] : v[h + j];
                        int o = hi ? op[h + j] : op[j];
                        P got = shfl_xor(give, off);
                        // the lower lane's value first, in both lanes' view
                        v[j] = hi ? red_combine(o, got, keep) : red_combine(o, keep, got);
                        op[j] = o;
                }
        }
        P r = v[0];
        int o = op[0];
#pragma unroll
        for (int off = 16 / KP; off > 0; off >>= 1)
                r = red_combine(o, r, shfl_down(r, off));
        return r;
}

// Block-wide reduction of K partials (double or DF); the totals, as
// doubles, land in out[0..K) (shared) and are visible to every thread of
// the block on return.
template <int K, class P>
__device__ __forceinline__ void block_reduce(const P (&v)[K], const int (&op)[K],
                                             double * out)
{
        constexpr int KP = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : 8;
        constexpr int G = 32 / KP;
        static_assert(K <= kRedMax, "at most kRedMax values per reduction");
        __shared__ P part[kWarp][kRedMax];
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        int nw = (blockDim.x + 31) >> 5;
        P w[KP];
        int o[KP];
#pragma unroll
        for (int k = 0; k < KP; k++) {
                o[k] = k < K ? op[k] : RED_SUM;
                w[k] = k < K ? v[k] : red_identity_as<P>(RED_SUM);
        }
        P r = warp_reduce_many<KP>(w, o, lane);
        if ((lane & (G - 1)) == 0 && lane / G < K)
                part[warp][lane / G] = r;
        __syncthreads();
        if (warp == 0) {
                // the warps' totals, lane q holding warp q's: the same butterfly
#pragma unroll
                for (int k = 0; k < KP; k++) {
                        o[k] = k < K ? op[k] : RED_SUM;
                        w[k] = (k < K && lane < nw) ? part[lane][k] : red_identity_as<P>(o[k]);
                }
                P t = warp_reduce_many<KP>(w, o, lane);
                if ((lane & (G - 1)) == 0 && lane / G < K)
                        out[lane / G] = to_double(t);
        }
        __syncthreads();
}

// Per-team control words in global memory (zeroed before the launch), each
// on its own 128-byte line.
struct alignas(128) CtlWord {
        unsigned v;
        unsigned pad[31];
};
// Phase timestamps of the grid team's reductions (optional): for the
// reductions first .. first + count - 1 (counted from 1 in each launch), CTA
// b's thread 0 records %globaltimer at kTracePhases points -- entering the
// reduction (its warp 0's share of the pass done), after the block
// reduction (the whole CTA done), and leaving it (every CTA's partials
// summed) -- at rec[((e - first) * gridDim.x + b) * kTracePhases + phase].
constexpr int kTracePhases = 3;
struct alignas(128) TraceBuf {
        unsigned long long * rec;  // nullptr: tracing off
        unsigned first, count;
};

struct TeamCtl {
        CtlWord status_w;
        // read by the grid team's thread 0 at each reduction, so tracing
        // costs the solve no registers
        TraceBuf trace;
};

// Reduction slots: per CTA and parity one 128-byte line of 16 64-bit words.
// Value k of a reduction is published as words 2k (low 32 bits of the
// double) and 2k + 1 (high 32 bits), each word carrying the reduction's
// epoch in its upper half: a reader that sees the current epoch in both
// words holds that value, with no separate tag and no second round trip
// (a naturally aligned 64-bit store is seen whole or not at all).
constexpr int kSlotStride = 16;  // words per line
// Lines a lane polls at once, per pass over the CTAs: 10 covers 320 CTAs
// (two per SM on 152 SMs) in one pass; more CTAs take further passes.
constexpr int kSumWidth = 10;
__device__ __forceinline__ ulonglong2 ld_relaxed_u64x2(const unsigned long long * p)
{
        ulonglong2 v;
        asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];"
                     : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
        return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu()
{
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long * p, unsigned long long v)
{
        asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

// Every CTA of a cooperative launch.  team.reduce() is an all-gather: each
// CTA publishes its partials in its own line (epoch-tagged words, see
// kSlotStride), then in every CTA warp k polls value k of all CTAs' lines
// until every word shows the current epoch and sums them in CTA order -- so
// every thread gets the same bits, about one L2 round trip after the last
// CTA publishes, with no counters.
template <bool Trace>
struct GridTeamT {
        TeamCtl * ctl;
        double * slots;   // [2][gridDim.x][kSlotStride] words
        double * result;  // unused (kept for the launch interface)
        int parity;
        unsigned epoch;   // reductions passed (the same count in every CTA)

        // (compiled into the traced kernel only: even an untaken branch here
        // costs the solve kernel registers)
        __device__ void stamp(unsigned e, int phase) const
        {
                if constexpr (Trace) if (threadIdx.x == 0) {
                        unsigned long long * rec = ctl->trace.rec;
                        if (rec) {
                                unsigned first = ctl->trace.first, i = e - first;
                                if (e >= first && i < ctl->trace.count)
                                        rec[((size_t)i * gridDim.x + blockIdx.x) * kTracePhases
                                            + phase] = global_ns();
                        }
                }
        }

        static constexpr bool kShared = false;
        static constexpr bool kStreamHint = false;  // see load_chunk

        __device__ int nthreads() const { return gridDim.x * blockDim.x; }
        __device__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
        __device__ int warp() const { return tid() >> 5; }
        __device__ int nwarps() const { return nthreads() >> 5; }

        // Loads of data other CTAs of the team write during the kernel go to
        // L2 (the L1 of another SM may hold a stale line).
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return __ldcg(p); }

        __device__ int * status() const
        {
                return reinterpret_cast<int *>(&ctl->status_w.v);
        }

        __device__ bool failed() const
        {
                return ld_acquire_int(status()) != 0;
        }

        __device__ void fail(int code)
        {
                atomicCAS(status(), 0, code);
        }

        // Reduction + barrier.  Returns false if the team has failed.
        template <int K, class P>
        __device__ bool reduce_to(const P (&v)[K], const int (&op)[K], double (&res)[K])
        {
                static_assert(2 * K <= kSlotStride, "two words per value in a line");
                __shared__ double tot[kRedMax];  // this CTA's totals
                __shared__ double fin[kRedMax];  // the team's
                __shared__ int bad[kRedMax];
                stamp(epoch + 1, 0);
                block_reduce<K>(v, op, tot);
                epoch++;
                stamp(epoch, 1);
                const unsigned nb = gridDim.x;
                unsigned long long * lines =
                        reinterpret_cast<unsigned long long *>(slots) + (size_t)parity * nb * kSlotStride;
                const unsigned long long tag = (unsigned long long)epoch << 32;
                if (threadIdx.x < 2 * K) {
                        unsigned long long bits =
                                (unsigned long long)__double_as_longlong(tot[threadIdx.x >> 1]);
                        unsigned half = (threadIdx.x & 1) ? (unsigned)(bits >> 32) : (unsigned)bits;
                        // release: this CTA's phase writes, ordered before
                        // this point by the block barrier
                        fence_acq_rel_gpu();
                        st_relaxed_u64(lines + (size_t)blockIdx.x * kSlotStride + threadIdx.x,
                                       tag | half);
                }
                int status_now = 0;
                if (threadIdx.x < 32 * K) {
                        // warp k: value k of every CTA, lanes taking CTAs
                        // lane, lane + 32, ...; combined in that fixed order,
                        // then a fixed shuffle tree
                        const int k = threadIdx.x >> 5, lane = threadIdx.x & 31;
                        const double idv = red_identity(op[k]);
                        double acc = idv;
                        int broke = 0;
                        unsigned long long t0 = 0;
                        for (unsigned base = 0; base < nb && !broke; base += 32u * kSumWidth) {
                                double vals[kSumWidth];
                                unsigned pending = 0;
#pragma unroll
                                for (int q = 0; q < kSumWidth; q++) {
                                        vals[q] = idv;
                                        if (base + lane + 32u * q < nb)
                                                pending |= 1u << q;
                                }
                                for (unsigned rounds = 0;; rounds++) {
                                        ulonglong2 w[kSumWidth];
#pragma unroll
                                        for (int q = 0; q < kSumWidth; q++) {
                                                unsigned b = base + lane + 32u * q;
                                                w[q] = ((pending >> q) & 1u)
                                                        ? ld_relaxed_u64x2(lines + (size_t)b * kSlotStride + 2 * k)
                                                        : make_ulonglong2(0, 0);
                                        }
#pragma unroll
                                        for (int q = 0; q < kSumWidth; q++) {
                                                if (((pending >> q) & 1u) &&
                                                    (w[q].x & 0xffffffff00000000ull) == tag &&
                                                    (w[q].y & 0xffffffff00000000ull) == tag) {
                                                        pending &= ~(1u << q);
                                                        vals[q] = __longlong_as_double(
                                                                (long long)((w[q].y << 32) | (w[q].x & 0xffffffffull)));
                                                }
                                        }
                                        if (!__any_sync(0xffffffffu, pending != 0))
                                                break;
                                        __nanosleep(16);
                                        if ((rounds & 63) == 63) {
                                                if (lane == 0) {
                                                        if (t0 == 0)
                                                                t0 = global_ns();
                                                        if (ld_acquire_int(status()) != 0)
                                                                broke = 1;
                                                        else if (global_ns() - t0 > kWaitLimitNs) {
                                                                fail(kStatusTimeout);
                                                                broke = 1;
                                                        }
                                                }
                                                broke = __shfl_sync(0xffffffffu, broke, 0);
                                                if (broke)
                                                        break;
                                        }
                                }
#pragma unroll
                                for (int q = 0; q < kSumWidth; q++)
                                        acc = red_combine(op[k], acc, vals[q]);
                        }
                        // acquire: the other CTAs' phase writes
                        fence_acq_rel_gpu();
                        acc = warp_reduce(acc, op[k]);
                        if (lane == 0) {
                                fin[k] = acc;
                                bad[k] = broke;
                        }
                        // the team's status word, alongside (a relaxed load:
                        // it only has to show a failure eventually)
                        if (threadIdx.x == 0)
                                status_now = ld_relaxed_int(status());
                }
                int b = __syncthreads_or(threadIdx.x == 0 && status_now != 0);
#pragma unroll
                for (int k = 0; k < K; k++) {
                        res[k] = fin[k];
                        b |= bad[k];
                }
                stamp(epoch, 2);
                parity ^= 1;
                return !b;
        }

        // In-place form for double partials.
        template <int K>
        __device__ bool reduce(double (&v)[K], const int (&op)[K])
        {
                return reduce_to<K, double>(v, op, v);
        }

        __device__ bool sync()
        {
                double d[1] = {0};
                const int op[1] = {RED_SUM};
                return reduce<1>(d, op);
        }
};

using GridTeam = GridTeamT<false>;

// One CTA (one LP of a batch): barriers are __syncthreads, reductions stay
// in shared memory, loads may use L1 (only this SM writes the LP's data).
struct BlockTeam {
        int * status;     // the LP's status word in global memory

        static constexpr bool kShared = true;
        static constexpr bool kStreamHint = false;  // see load_chunk

        __device__ int nthreads() const { return blockDim.x; }
        __device__ int tid() const { return threadIdx.x; }
        __device__ int warp() const { return threadIdx.x >> 5; }
        __device__ int nwarps() const { return blockDim.x >> 5; }
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return *p; }
        __device__ bool failed() const { return *(volatile int *)status != 0; }
        __device__ void fail(int code) { atomicCAS(status, 0, code); }

        // Failures of a one-CTA team are raised by its own threads, which
        // all return at once, so the reduction needs no status check.
        template <int K, class P>
        __device__ bool reduce_to(const P (&v)[K], const int (&op)[K], double (&res)[K])
        {
                __shared__ double tot[kRedMax];
                block_reduce<K>(v, op, tot);
#pragma unroll
                for (int k = 0; k < K; k++)
                        res[k] = tot[k];
                return true;
        }

        // In-place form for double partials.
        template <int K>
        __device__ bool reduce(double (&v)[K], const int (&op)[K])
        {
                return reduce_to<K, double>(v, op, v);
        }

        __device__ bool sync()
        {
                __syncthreads();
                return true;
        }
};

// The CTAs of one thread-block cluster (one large LP of a batch or a
// server): barriers are the hardware cluster barrier (release / acquire at
// cluster scope); each CTA publishes its partials in its own shared memory
// and every CTA sums all CTAs' partials, read through distributed shared
// memory, in rank order -- so every thread gets the same bits.
struct ClusterTeam {
        int * status;
        unsigned rank, size;
        int parity;

        static constexpr bool kShared = false;
        static constexpr bool kStreamHint = false;  // see load_chunk

        __device__ explicit ClusterTeam(int * st) : status(st), parity(0)
        {
                cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
                rank = cl.block_rank();
                size = cl.num_blocks();
        }

        __device__ int nthreads() const { return size * blockDim.x; }
        __device__ int tid() const { return rank * blockDim.x + threadIdx.x; }
        __device__ int warp() const { return tid() >> 5; }
        __device__ int nwarps() const { return nthreads() >> 5; }
        // data other CTAs of the cluster write: L2, not a possibly stale L1
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return __ldcg(p); }
        __device__ bool failed() const { return ld_acquire_int(status) != 0; }
        __device__ void fail(int code) { atomicCAS(status, 0, code); }

        // Failures are decided from reduced values, identically in every CTA,
        // so the reduction needs no status check.
        template <int K, class P>
        __device__ bool reduce_to(const P (&v)[K], const int (&op)[K], double (&res)[K])
        {
                __shared__ double part[2][kRedMax];
                __shared__ double tot[kRedMax];
                block_reduce<K>(v, op, tot);
                if (threadIdx.x < K)
                        part[parity][threadIdx.x] = tot[threadIdx.x];
                cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
                cl.sync();
                int lane = threadIdx.x & 31, wk = threadIdx.x >> 5;
#pragma unroll
                for (int k = 0; k < K; k++) {
                        if (wk != k)
                                continue;
                        double val = red_identity(op[k]);
                        if ((unsigned)lane < size)
                                val = *cl.map_shared_rank(&part[parity][k], lane);
                        val = warp_reduce(val, op[k]);
                        if (lane == 0)
                                tot[k] = val;
                }
                __syncthreads();
#pragma unroll
                for (int k = 0; k < K; k++)
                        res[k] = tot[k];
                parity ^= 1;
                return true;
        }

        // In-place form for double partials.
        template <int K>
        __device__ bool reduce(double (&v)[K], const int (&op)[K])
        {
                return reduce_to<K, double>(v, op, v);
        }

        __device__ bool sync()
        {
                cooperative_groups::this_cluster().sync();
                return true;
        }
};

// A SELL operator on the device (layout.h: Sell).  Slice s starts at
// element ptr[s] & ~31 and holds 32 >> c rows from row0[s], each spread over
// L = 1 << c lanes, c = ptr[s] & 7; per step a lane reads V consecutive
// entries of its row: V = 4 (one int4 of columns, one float4 or two double2
// of values) when bit 3 of ptr[s] is set, else V = 1.
template <class V>
struct SellDev {
        int nrows;
        int nslices;
        const int64_t * ptr;
        const int32_t * row0;
        const int32_t * col;
        const V * val;
};

// One warp's view of one slice.
struct Slice {
        int64_t base;   // first element
        int steps;      // steps (32 V elements each)
        int shift;      // log2(lanes per row)
        bool vec;       // V = 4
        int row;        // this lane's row (may be >= nrows: padding)
        bool lead;      // this lane owns its row's result
};

__device__ __forceinline__ Slice slice_from(int64_t p0, int64_t p1, int row0, int lane)
{
        Slice sl;
        sl.shift = (int)(p0 & 7);
        sl.vec = (p0 & 8) != 0;
        sl.base = p0 & ~int64_t(31);
        sl.steps = (int)(((p1 & ~int64_t(31)) - sl.base) >> (sl.vec ? 7 : 5));
        sl.row = row0 + (lane >> sl.shift);
        sl.lead = (lane & ((1 << sl.shift) - 1)) == 0;
        return sl;
}

template <class V>
__device__ __forceinline__ Slice slice_of(const SellDev<V> & op, int s, int lane)
{
        return slice_from(__ldg(op.ptr + s), __ldg(op.ptr + s + 1), __ldg(op.row0 + s), lane);
}

// Entries per lane per step, as a type (for generic lambdas).
template <int N>
struct VecW {
        static constexpr int value = N;
};

// Runs f(VecW<4>) on a vector slice, f(VecW<1>) on a scalar one.
template <class F>
__device__ __forceinline__ auto by_width(const Slice & sl, F && f) -> decltype(f(VecW<1>()))
{
        if (sl.vec)
                return f(VecW<4>());
        return f(VecW<1>());
}

// One lane's VEC entries of one step: columns and values.
template <int VEC, class V>
struct Chunk {
        int c[VEC];
        V a[VEC];
};

// An L2 policy that evicts the lines it tags first: a matrix streamed once
// through a product far larger than L2 should not push out the gathered
// vector, which every row reuses.
__device__ __forceinline__ unsigned long long evict_first_policy()
{
        unsigned long long p;
        asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
        return p;
}

__device__ __forceinline__ int ld_stream(const int32_t * p, unsigned long long pol)
{
        int r;
        asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
        return r;
}
__device__ __forceinline__ double ld_stream(const double * p, unsigned long long pol)
{
        double r;
        asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(r) : "l"(p), "l"(pol));
        return r;
}
__device__ __forceinline__ float ld_stream(const float * p, unsigned long long pol)
{
        float r;
        asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
        return r;
}
__device__ __forceinline__ int4 ld_stream_v4(const int32_t * p, unsigned long long pol)
{
        int4 r;
        asm("ld.global.nc.L2::cache_hint.v4.s32 {%0, %1, %2, %3}, [%4], %5;"
            : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
            : "l"(p), "l"(pol));
        return r;
}
__device__ __forceinline__ double2 ld_stream_v2(const double * p, unsigned long long pol)
{
        double2 r;
        asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
            : "=d"(r.x), "=d"(r.y)
            : "l"(p), "l"(pol));
        return r;
}
__device__ __forceinline__ float4 ld_stream_v4(const float * p, unsigned long long pol)
{
        float4 r;
        asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
            : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
            : "l"(p), "l"(pol));
        return r;
}

// The matrix entries of one step, tagged evict-first in L2 when `pol` is
// nonzero (a team that streams a matrix once, kStreamHint), plain
// read-only loads otherwise (a solve's team keeps its matrix in L2 across
// iterations).
template <int VEC, class V>
__device__ __forceinline__ Chunk<VEC, V> load_chunk_hinted(const int32_t * col, const V * val,
                                                           int64_t at, unsigned long long pol)
{
        Chunk<VEC, V> q;
        if constexpr (VEC == 1) {
                q.c[0] = ld_stream(col + at, pol);
                q.a[0] = ld_stream(val + at, pol);
        } else {
                static_assert(VEC == 4, "vector slices hold 4 entries per lane");
                int4 c = ld_stream_v4(col + at, pol);
                q.c[0] = c.x;
                q.c[1] = c.y;
                q.c[2] = c.z;
                q.c[3] = c.w;
                if constexpr (sizeof(V) == 8) {
                        double2 a = ld_stream_v2(val + at, pol);
                        double2 b = ld_stream_v2(val + at + 2, pol);
                        q.a[0] = a.x;
                        q.a[1] = a.y;
                        q.a[2] = b.x;
                        q.a[3] = b.y;
                } else {
                        float4 a = ld_stream_v4(val + at, pol);
                        q.a[0] = a.x;
                        q.a[1] = a.y;
                        q.a[2] = a.z;
                        q.a[3] = a.w;
                }
        }
        return q;
}

template <int VEC, class Team, class V>
__device__ __forceinline__ Chunk<VEC, V> team_chunk(const Team & tm, const int32_t * col,
                                                    const V * val, int64_t at);

template <int VEC, class V>
__device__ __forceinline__ Chunk<VEC, V> load_chunk(const int32_t * col, const V * val,
                                                    int64_t at)
{
        Chunk<VEC, V> q;
        if constexpr (VEC == 1) {
                q.c[0] = __ldg(col + at);
                q.a[0] = __ldg(val + at);
        } else {
                static_assert(VEC == 4, "vector slices hold 4 entries per lane");
                int4 c = __ldg(reinterpret_cast<const int4 *>(col + at));
                q.c[0] = c.x;
                q.c[1] = c.y;
                q.c[2] = c.z;
                q.c[3] = c.w;
                if constexpr (sizeof(V) == 8) {
                        double2 a = __ldg(reinterpret_cast<const double2 *>(val + at));
                        double2 b = __ldg(reinterpret_cast<const double2 *>(val + at + 2));
                        q.a[0] = a.x;
                        q.a[1] = a.y;
                        q.a[2] = b.x;
                        q.a[3] = b.y;
                } else {
                        float4 a = __ldg(reinterpret_cast<const float4 *>(val + at));
                        q.a[0] = a.x;
                        q.a[1] = a.y;
                        q.a[2] = a.z;
                        q.a[3] = a.w;
                }
        }
        return q;
}

// The step loads of a team: evict-first for teams that stream (kStreamHint,
// with their policy in tm.policy).
template <int VEC, class Team, class V>
__device__ __forceinline__ Chunk<VEC, V> team_chunk(const Team & tm, const int32_t * col,
                                                    const V * val, int64_t at)
{
        if constexpr (Team::kStreamHint)
                return load_chunk_hinted<VEC>(col, val, at, tm.policy);
        else
                return load_chunk<VEC>(col, val, at);
}

// Visits slices so each warp of the team gets a balanced share: slices come
// in decreasing width, and are dealt in snake order (0..W-1, W-1..0, ...).
template <class Team, class F>
__device__ __forceinline__ void for_each_slice(const Team & tm, int nslices, F && f)
{
        int w = tm.warp(), W = tm.nwarps();
        for (int round = 0;; round++) {
                int s = round * W + ((round & 1) ? W - 1 - w : w);
                if (round * W >= nslices)
                        break;
                if (s < nslices)
                        f(s);
        }
}

// The same walk over the slices of one operator, handing f the decoded
// slice; the next slice's words are loaded while f works on the current
// one (a warp handles only a few slices per pass, so the load latency of
// each slice's header would otherwise be exposed).
template <class Team, class V, class F>
__device__ __forceinline__ void for_each_slice_of(const Team & tm, const SellDev<V> & op,
                                                  int lane, F && f)
{
        int w = tm.warp(), W = tm.nwarps();
        const int ns = op.nslices;
        auto pick = [&](int round) { return round * W + ((round & 1) ? W - 1 - w : w); };
        int s = pick(0);
        int64_t p0 = 0, p1 = 0;
        int r0 = 0;
        if (s < ns) {
                p0 = __ldg(op.ptr + s);
                p1 = __ldg(op.ptr + s + 1);
                r0 = __ldg(op.row0 + s);
        }
        for (int round = 0; round * W < ns; round++) {
                int sn = pick(round + 1);
                int64_t q0 = 0, q1 = 0;
                int rn = 0;
                if (sn < ns) {
                        q0 = __ldg(op.ptr + sn);
                        q1 = __ldg(op.ptr + sn + 1);
                        rn = __ldg(op.row0 + sn);
                }
                if (s < ns)
                        f(slice_from(p0, p1, r0, lane));
                s = sn;
                p0 = q0;
                p1 = q1;
                r0 = rn;
        }
}

// Sum of the L = 1 << shift lanes of each row group, into its first lane, by
// a fixed tree.
template <class T>
__device__ __forceinline__ T lanes_tree(T v, int shift)
{
        for (int o = (1 << shift) >> 1; o > 0; o >>= 1)
                v += __shfl_down_sync(0xffffffffu, v, o, 1 << shift);
        return v;
}

__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double mul_exact(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_exact(float a, float b) { return __fmul_rn(a, b); }

// acc (valid in each group's first lane) += the group's V L terms of one
// step, in row order (lane by lane, V each), every addition rounded: the
// sequential order of the row.
template <int VEC, class T>
__device__ __forceinline__ T in_order(T acc, const T (&p)[VEC], int shift, int lane)
{
        if (shift == 0) {
#pragma unroll
                for (int j = 0; j < VEC; j++)
                        acc = add_rn(acc, p[j]);
                return acc;
        }
        int L = 1 << shift, first = lane & ~(L - 1);
        for (int q = 0; q < L; q++) {
#pragma unroll
                for (int j = 0; j < VEC; j++)
                        acc = add_rn(acc, __shfl_sync(0xffffffffu, p[j], first + q));
        }
        return acc;
}

// Multiply-add used by the row sums: fused (default) or the reference's
// separate rounding of product and sum (Exact), which reproduces its bits.
template <bool Exact>
__device__ __forceinline__ double madd(double a, double b, double c)
{
        if (Exact)
                return __dadd_rn(c, __dmul_rn(a, b));
        return fma(a, b, c);
}

template <bool Exact>
__device__ __forceinline__ float madd(float a, float b, float c)
{
        if (Exact)
                return __fadd_rn(c, __fmul_rn(a, b));
        return fmaf(a, b, c);
}

// Rows longer than this, in FP32, combine their lanes' partial sums in FP64
// (a compensated sum of the row).
constexpr int kCompensateWidth = 256;

// Finishes a row sum held as per-lane partials with a fixed tree; `width`
// is the row capacity of the slice.
template <class T>
__device__ __forceinline__ T finish_row(T acc, int shift, int width)
{
        if (shift == 0)
                return acc;
        if (sizeof(T) == 4 && width > kCompensateWidth)
                return (T)lanes_tree((double)acc, shift);
        return lanes_tree(acc, shift);
}

// One row sum of a SELL slice: sum_k A_k x[col_k] for the row of this lane
// (valid in the row's lead lane).  Exact: the row's sequential order with
// rounded products and sums; otherwise FMA chains per lane and a tree.
template <bool Exact, int VEC, int XS, class Team, class V, class T>
__device__ __forceinline__ T slice_row_sum(const Team & tm, const SellDev<V> & op,
                                           const Slice & sl, const T * x, int lane)
{
        int64_t at = sl.base + VEC * lane;
        T acc = 0;
        if constexpr (Exact) {
                for (int t = 0; t < sl.steps; t++, at += 32 * VEC) {
                        Chunk<VEC, V> q = team_chunk<VEC>(tm, op.col, op.val, at);
                        T p[VEC];
#pragma unroll
                        for (int j = 0; j < VEC; j++)
                                p[j] = mul_exact((T)q.a[j], tm.ld(x + XS * q.c[j]));
                        acc = in_order<VEC>(acc, p, sl.shift, lane);
                }
                return acc;
        } else {
                T acc2 = 0;
                int t = 0;
                for (; t + 2 <= sl.steps; t += 2, at += 64 * VEC) {
                        Chunk<VEC, V> q0 = team_chunk<VEC>(tm, op.col, op.val, at);
                        Chunk<VEC, V> q1 = team_chunk<VEC>(tm, op.col, op.val, at + 32 * VEC);
                        T x0[VEC], x1[VEC];
#pragma unroll
                        for (int j = 0; j < VEC; j++) {
                                x0[j] = tm.ld(x + XS * q0.c[j]);
                                x1[j] = tm.ld(x + XS * q1.c[j]);
                        }
#pragma unroll
                        for (int j = 0; j < VEC; j++) {
                                acc = madd<false>((T)q0.a[j], x0[j], acc);
                                acc2 = madd<false>((T)q1.a[j], x1[j], acc2);
                        }
                }
                if (t < sl.steps) {
                        Chunk<VEC, V> q0 = team_chunk<VEC>(tm, op.col, op.val, at);
#pragma unroll
                        for (int j = 0; j < VEC; j++)
                                acc = madd<false>((T)q0.a[j], tm.ld(x + XS * q0.c[j]), acc);
                }
                return finish_row(acc + acc2, sl.shift, (sl.steps * VEC) << sl.shift);
        }
}

// Row sums of one SELL operator applied to x (entry j of x at x[XS j]).
// For every live row, in the row's lead lane: pv = pre(row) is loaded
// before the row's entries (so the epilogue's operands arrive while the row
// is summed), then epi(row, sum, pv).
template <bool Exact, int XS = 1, class Team, class V, class T, class Pre, class Epi>
__device__ __forceinline__ void sell_rows_1p(const Team & tm, const SellDev<V> & op,
                                             const T * x, Pre && pre, Epi && epi)
{
        int lane = threadIdx.x & 31;
        for_each_slice_of(tm, op, lane, [&](const Slice & sl) {
                bool live = sl.lead && sl.row < op.nrows;
                auto pv = pre(live ? sl.row : -1);
                T acc = by_width(sl, [&](auto w) {
                        return slice_row_sum<Exact, decltype(w)::value, XS>(tm, op, sl, x, lane);
                });
                if (live)
                        epi(sl.row, acc, pv);
        });
}

struct NoPre {
        __device__ int operator()(int) const { return 0; }
};

// Row sums of one SELL operator applied to x (entry j at x[XS j]); calls
// epi(row, sum) in the row's lead lane for every live row.
template <bool Exact, int XS = 1, class Team, class V, class T, class Epi>
__device__ __forceinline__ void sell_rows_1(const Team & tm, const SellDev<V> & op,
                                            const T * x, Epi && epi)
{
        sell_rows_1p<Exact, XS>(tm, op, x, NoPre(), [&](int r, T acc, int) { epi(r, acc); });
}

// Two right-hand sides sharing one pass over the operator, with the same
// pre / epi protocol as sell_rows_1p: epi(row, sum0, sum1, pv).
template <bool Exact, class Team, class V, class T, class Pre, class Epi>
__device__ __forceinline__ void sell_rows_2p(const Team & tm, const SellDev<V> & op,
                                             const T * x0, const T * x1, Pre && pre,
                                             Epi && epi)
{
        int lane = threadIdx.x & 31;
        for_each_slice_of(tm, op, lane, [&](const Slice & sl) {
                bool live = sl.lead && sl.row < op.nrows;
                auto pv = pre(live ? sl.row : -1);
                T a0 = 0, a1 = 0;
                by_width(sl, [&](auto w) {
                        constexpr int VEC = decltype(w)::value;
                        int64_t at = sl.base + VEC * lane;
                        for (int t = 0; t < sl.steps; t++, at += 32 * VEC) {
                                Chunk<VEC, V> q = team_chunk<VEC>(tm, op.col, op.val, at);
                                T p[VEC], r[VEC];
#pragma unroll
                                for (int j = 0; j < VEC; j++) {
                                        p[j] = tm.ld(x0 + q.c[j]);
                                        r[j] = tm.ld(x1 + q.c[j]);
                                }
                                if constexpr (Exact) {
#pragma unroll
                                        for (int j = 0; j < VEC; j++) {
                                                p[j] = mul_exact((T)q.a[j], p[j]);
                                                r[j] = mul_exact((T)q.a[j], r[j]);
                                        }
                                        a0 = in_order<VEC>(a0, p, sl.shift, lane);
                                        a1 = in_order<VEC>(a1, r, sl.shift, lane);
                                } else {
#pragma unroll
                                        for (int j = 0; j < VEC; j++) {
                                                a0 = madd<false>((T)q.a[j], p[j], a0);
                                                a1 = madd<false>((T)q.a[j], r[j], a1);
                                        }
                                }
                        }
                        if constexpr (!Exact) {
                                int width = (sl.steps * VEC) << sl.shift;
                                a0 = finish_row(a0, sl.shift, width);
                                a1 = finish_row(a1, sl.shift, width);
                        }
                        return 0;
                });
                if (live)
                        epi(sl.row, a0, a1, pv);
        });
}

template <bool Exact, class Team, class V, class T, class Epi>
__device__ __forceinline__ void sell_rows_2(const Team & tm, const SellDev<V> & op,
                                            const T * x0, const T * x1, Epi && epi)
{
        sell_rows_2p<Exact>(tm, op, x0, x1, NoPre(),
                            [&](int r, T a0, T a1, int) { epi(r, a0, a1); });
}

// Two values stored side by side (16 bytes for doubles, 8 for floats).
template <class T>
struct PairOf;
template <>
struct PairOf<double> {
        typedef double2 type;
};
template <>
struct PairOf<float> {
        typedef float2 type;
};

// p[0] = a, p[1] = b in one store (p aligned to the pair's size).
template <class T>
__device__ __forceinline__ void store_pair(T * p, T a, T b)
{
        typedef typename PairOf<T>::type P2;
        P2 v;
        v.x = a;
        v.y = b;
        *reinterpret_cast<P2 *>(p) = v;
}

// Two right-hand sides stored as one interleaved pair vector (entry j of the
// first at xy[2 j], of the second at xy[2 j + 1]; xy aligned to a pair):
// each entry of the operator fetches both with one gather.  Same sums and
// the same pre / epi protocol as sell_rows_2p: epi(row, sum0, sum1, pv).
template <bool Exact, class Team, class V, class T, class Pre, class Epi>
__device__ __forceinline__ void sell_rows_pair(const Team & tm, const SellDev<V> & op,
                                               const T * xy, Pre && pre, Epi && epi)
{
        typedef typename PairOf<T>::type P2;
        const P2 * xp = reinterpret_cast<const P2 *>(xy);
        int lane = threadIdx.x & 31;
        for_each_slice_of(tm, op, lane, [&](const Slice & sl) {
                bool live = sl.lead && sl.row < op.nrows;
                auto pv = pre(live ? sl.row : -1);
                T a0 = 0, a1 = 0;
                by_width(sl, [&](auto w) {
                        constexpr int VEC = decltype(w)::value;
                        int64_t at = sl.base + VEC * lane;
                        if constexpr (Exact) {
                                for (int t = 0; t < sl.steps; t++, at += 32 * VEC) {
                                        Chunk<VEC, V> q = team_chunk<VEC>(tm, op.col, op.val, at);
                                        T p[VEC], r[VEC];
#pragma unroll
                                        for (int j = 0; j < VEC; j++) {
                                                P2 g = tm.ld(xp + q.c[j]);
                                                p[j] = mul_exact((T)q.a[j], g.x);
                                                r[j] = mul_exact((T)q.a[j], g.y);
                                        }
                                        a0 = in_order<VEC>(a0, p, sl.shift, lane);
                                        a1 = in_order<VEC>(a1, r, sl.shift, lane);
                                }
                        } else {
                                for (int t = 0; t < sl.steps; t++, at += 32 * VEC) {
                                        Chunk<VEC, V> q = team_chunk<VEC>(tm, op.col, op.val, at);
                                        P2 g[VEC];
#pragma unroll
                                        for (int j = 0; j < VEC; j++)
                                                g[j] = tm.ld(xp + q.c[j]);
#pragma unroll
                                        for (int j = 0; j < VEC; j++) {
                                                a0 = madd<false>((T)q.a[j], g[j].x, a0);
                                                a1 = madd<false>((T)q.a[j], g[j].y, a1);
                                        }
                                }
                                int width = (sl.steps * VEC) << sl.shift;
                                a0 = finish_row(a0, sl.shift, width);
                                a1 = finish_row(a1, sl.shift, width);
                        }
                        return 0;
                });
                if (live)
                        epi(sl.row, a0, a1, pv);
        });
}

}  // namespace acd
