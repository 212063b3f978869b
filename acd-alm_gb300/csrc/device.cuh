// Device primitives shared by the kernels: teams of threads that run one
// solve together, deterministic reductions, bounded waits, SELL row loops.
//
// A "team" is the set of threads that cooperate on one LP.  Every thread of
// a team executes the same control flow (the solver's scalars are computed
// redundantly from identical reduction results), data-parallel phases split
// rows over the team's warps, and team.reduce() is both the reduction and
// the barrier between phases.
//
//   GridTeam  - every CTA of a cooperative launch (one large LP).  The
//               barrier is a counter + generation word in global memory; the
//               last CTA to arrive sums the per-CTA partials in CTA order and
//               publishes the totals, so every CTA reads the same bits.
//   BlockTeam - one CTA (one small LP of a batch); __syncthreads based.
//
// No wait is unbounded: a CTA that waits more than kWaitLimitNs for the
// others records ACDALM_ETIMEOUT in the team's status word and every thread
// returns; nothing traps.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace acd {

constexpr int kWarp = 32;
constexpr int kRedMax = 8;                           // values per reduction
constexpr unsigned long long kWaitLimitNs = 20ull * 1000000000ull;
constexpr int kStatusTimeout = -2;                   // ACDALM_ETIMEOUT
constexpr int kStatusNonFinite = -5;                 // ACDALM_ENONFINITE

enum RedOp { RED_SUM = 0, RED_MAX = 1, RED_MIN = 2 };

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

__device__ __forceinline__ int ld_acquire_int(const int * p)
{
        int v;
        asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p)
                     : "memory");
        return v;
}

// Lane 0 of each warp ends with the warp's combination (fixed tree order).
__device__ __forceinline__ double warp_reduce(double v, int op)
{
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
                v = red_combine(op, v, __shfl_down_sync(0xffffffffu, v, o));
        return v;
}

// Block-wide reduction of K values; the totals land in out[0..K) (shared)
// and are visible to every thread of the block on return.
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], const int (&op)[K],
                                             double * out)
{
        __shared__ double part[kWarp][kRedMax];
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int k = 0; k < K; k++) {
                double r = warp_reduce(v[k], op[k]);
                if (lane == 0)
                        part[warp][k] = r;
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
                for (int k = 0; k < K; k++) {
                        double r = (lane < nw) ? part[lane][k]
                                               : red_identity(op[k]);
                        r = warp_reduce(r, op[k]);
                        if (lane == 0)
                                out[k] = r;
                }
        }
        __syncthreads();
}

// Per-team control words in global memory (zeroed before the launch).
struct TeamCtl {
        unsigned count;
        unsigned gen;
        int status;
        int pad;
};

struct GridTeam {
        TeamCtl * ctl;
        double * slots;   // [2][gridDim.x][kRedMax]
        double * result;  // [2][kRedMax]
        int parity;

        static constexpr bool kShared = false;

        __device__ int nthreads() const { return gridDim.x * blockDim.x; }
        __device__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
        __device__ int warp() const { return tid() >> 5; }
        __device__ int nwarps() const { return nthreads() >> 5; }

        // Loads of data other CTAs of the team write during the kernel go to
        // L2 (the L1 of another SM may hold a stale line).
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return __ldcg(p); }

        __device__ bool failed() const
        {
                return ld_acquire_int(&ctl->status) != 0;
        }

        __device__ void fail(int code)
        {
                atomicCAS(&ctl->status, 0, code);
        }

        // Reduction + barrier.  Returns false if the team has failed.
        template <int K>
        __device__ bool reduce(double (&v)[K], const int (&op)[K])
        {
                __shared__ double tot[kRedMax];
                __shared__ int last;
                __shared__ unsigned gen0;
                __shared__ int bad;
                block_reduce<K>(v, op, tot);
                double * mine = slots
                        + ((size_t)parity * gridDim.x + blockIdx.x) * kRedMax;
                if (threadIdx.x < K)
                        __stcg(mine + threadIdx.x, tot[threadIdx.x]);
                __syncthreads();
                if (threadIdx.x == 0) {
                        __threadfence();
                        gen0 = ld_acquire(&ctl->gen);
                        unsigned prev = atomicAdd(&ctl->count, 1u);
                        last = (prev == gridDim.x - 1);
                }
                __syncthreads();
                if (last) {
                        if (threadIdx.x < 32) {
                                int lane = threadIdx.x;
                                const double * base = slots
                                        + (size_t)parity * gridDim.x * kRedMax;
#pragma unroll
                                for (int k = 0; k < K; k++) {
                                        double acc = red_identity(op[k]);
                                        for (unsigned b = lane; b < gridDim.x; b += 32)
                                                acc = red_combine(op[k], acc,
                                                                  __ldcg(base + (size_t)b * kRedMax + k));
                                        acc = warp_reduce(acc, op[k]);
                                        if (lane == 0)
                                                __stcg(result + parity * kRedMax + k, acc);
                                }
                                __syncwarp();
                                if (lane == 0) {
                                        __threadfence();
                                        atomicExch(&ctl->count, 0u);
                                        __threadfence();
                                        atomicAdd(&ctl->gen, 1u);
                                }
                        }
                } else if (threadIdx.x == 0) {
                        unsigned long long t0 = global_ns();
                        unsigned spins = 0;
                        while (ld_acquire(&ctl->gen) == gen0) {
                                __nanosleep(32);
                                if ((++spins & 255) == 0) {
                                        if (ld_acquire_int(&ctl->status) != 0)
                                                break;
                                        if (global_ns() - t0 > kWaitLimitNs) {
                                                fail(kStatusTimeout);
                                                break;
                                        }
                                }
                        }
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                        __threadfence();
                        bad = ld_acquire_int(&ctl->status) != 0;
                }
                if (threadIdx.x < K)
                        tot[threadIdx.x] = __ldcg(result + parity * kRedMax + threadIdx.x);
                __syncthreads();
#pragma unroll
                for (int k = 0; k < K; k++)
                        v[k] = tot[k];
                parity ^= 1;
                return !bad;
        }

        __device__ bool sync()
        {
                double d[1] = {0};
                const int op[1] = {RED_SUM};
                return reduce<1>(d, op);
        }
};

struct BlockTeam {
        int * status;     // per-instance status word in global memory
        static constexpr bool kShared = true;

        __device__ int nthreads() const { return blockDim.x; }
        __device__ int tid() const { return threadIdx.x; }
        __device__ int warp() const { return threadIdx.x >> 5; }
        __device__ int nwarps() const { return blockDim.x >> 5; }
        template <class T>
        __device__ __forceinline__ T ld(const T * p) const { return *p; }
        __device__ bool failed() const { return *(volatile int *)status != 0; }
        __device__ void fail(int code) { atomicCAS(status, 0, code); }

        template <int K>
        __device__ bool reduce(double (&v)[K], const int (&op)[K])
        {
                __shared__ double tot[kRedMax];
                __shared__ int bad;
                block_reduce<K>(v, op, tot);
#pragma unroll
                for (int k = 0; k < K; k++)
                        v[k] = tot[k];
                if (threadIdx.x == 0)
                        bad = *(volatile int *)status != 0;
                __syncthreads();
                int b = bad;
                __syncthreads();
                return !b;
        }

        __device__ bool sync()
        {
                __syncthreads();
                return true;
        }
};

// A SELL operator on the device: slice s holds rows [32s, 32s+32), element
// (lane r, slot k) at ptr[s] + 32k + r.
template <class V>
struct SellDev {
        int nrows;
        int nslices;
        const int64_t * ptr;
        const int32_t * col;
        const V * val;
};

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

// Long rows (more than this many nonzeros) in FP32 accumulate with a
// compensated (two-sum) sum.
constexpr int kCompensateWidth = 256;

template <class T>
struct Acc {
        T s, c;
        __device__ __forceinline__ void init() { s = 0; c = 0; }
};

// Row sums of one SELL operator applied to x (one lane per row); calls
// epi(row, sum) for every live row.  Rows are visited slice by slice, the
// team's warps taking slices round-robin.
template <bool Exact, class Team, class V, class T, class Epi>
__device__ __forceinline__ void sell_rows_1(const Team & tm, const SellDev<V> & op,
                                            const T * x, Epi && epi)
{
        int lane = threadIdx.x & 31;
        for (int s = tm.warp(); s < op.nslices; s += tm.nwarps()) {
                int64_t base = op.ptr[s];
                int w = (int)((op.ptr[s + 1] - base) >> 5);
                const int32_t * cp = op.col + base + lane;
                const V * vp = op.val + base + lane;
                T acc = 0;
                if (sizeof(T) == 4 && w > kCompensateWidth) {
                        T comp = 0;
                        for (int k = 0; k < w; k++) {
                                T prod = (T)__ldg(vp + 32 * k) * tm.ld(x + __ldg(cp + 32 * k));
                                T y = prod - comp;
                                T t = acc + y;
                                comp = (t - acc) - y;
                                acc = t;
                        }
                } else {
                        int k = 0;
                        for (; k + 4 <= w; k += 4) {
                                int c0 = __ldg(cp + 32 * k), c1 = __ldg(cp + 32 * (k + 1)),
                                    c2 = __ldg(cp + 32 * (k + 2)), c3 = __ldg(cp + 32 * (k + 3));
                                T v0 = (T)__ldg(vp + 32 * k), v1 = (T)__ldg(vp + 32 * (k + 1)),
                                  v2 = (T)__ldg(vp + 32 * (k + 2)), v3 = (T)__ldg(vp + 32 * (k + 3));
                                T x0 = tm.ld(x + c0), x1 = tm.ld(x + c1),
                                  x2 = tm.ld(x + c2), x3 = tm.ld(x + c3);
                                acc = madd<Exact>(v0, x0, acc);
                                acc = madd<Exact>(v1, x1, acc);
                                acc = madd<Exact>(v2, x2, acc);
                                acc = madd<Exact>(v3, x3, acc);
                        }
                        for (; k < w; k++)
                                acc = madd<Exact>((T)__ldg(vp + 32 * k),
                                                  tm.ld(x + __ldg(cp + 32 * k)), acc);
                }
                int row = s * 32 + lane;
                if (row < op.nrows)
                        epi(row, acc);
        }
}

// Two right-hand sides sharing one pass over the operator.
template <bool Exact, class Team, class V, class T, class Epi>
__device__ __forceinline__ void sell_rows_2(const Team & tm, const SellDev<V> & op,
                                            const T * x0, const T * x1, Epi && epi)
{
        int lane = threadIdx.x & 31;
        for (int s = tm.warp(); s < op.nslices; s += tm.nwarps()) {
                int64_t base = op.ptr[s];
                int w = (int)((op.ptr[s + 1] - base) >> 5);
                const int32_t * cp = op.col + base + lane;
                const V * vp = op.val + base + lane;
                T a0 = 0, a1 = 0;
                if (sizeof(T) == 4 && w > kCompensateWidth) {
                        T c0 = 0, c1 = 0;
                        for (int k = 0; k < w; k++) {
                                int c = __ldg(cp + 32 * k);
                                T v = (T)__ldg(vp + 32 * k);
                                T y0 = v * tm.ld(x0 + c) - c0, t0 = a0 + y0;
                                c0 = (t0 - a0) - y0;
                                a0 = t0;
                                T y1 = v * tm.ld(x1 + c) - c1, t1 = a1 + y1;
                                c1 = (t1 - a1) - y1;
                                a1 = t1;
                        }
                } else {
                        int k = 0;
                        for (; k + 2 <= w; k += 2) {
                                int c0 = __ldg(cp + 32 * k), c1 = __ldg(cp + 32 * (k + 1));
                                T v0 = (T)__ldg(vp + 32 * k), v1 = (T)__ldg(vp + 32 * (k + 1));
                                T p0 = tm.ld(x0 + c0), q0 = tm.ld(x1 + c0);
                                T p1 = tm.ld(x0 + c1), q1 = tm.ld(x1 + c1);
                                a0 = madd<Exact>(v0, p0, a0);
                                a1 = madd<Exact>(v0, q0, a1);
                                a0 = madd<Exact>(v1, p1, a0);
                                a1 = madd<Exact>(v1, q1, a1);
                        }
                        for (; k < w; k++) {
                                int c = __ldg(cp + 32 * k);
                                T v = (T)__ldg(vp + 32 * k);
                                a0 = madd<Exact>(v, tm.ld(x0 + c), a0);
                                a1 = madd<Exact>(v, tm.ld(x1 + c), a1);
                        }
                }
                int row = s * 32 + lane;
                if (row < op.nrows)
                        epi(row, a0, a1);
        }
}

}  // namespace acd
