// The APPROX inner solver and the ALM outer loop as device code, run by one
// team of threads per LP (see device.cuh).  The control flow, the caching of
// violations and values, and every stopping rule follow the reference:
// approx/approx.c:328-708 (iter, try_long_step, short_step, approx_solve),
// approx/step_project.inc, approx/gradient_value.inc, approx/vector.inc and
// alm.c:106-322.  Each pass over A or A' is one phase; the vector work that
// the reference does in separate loops (prox step, momentum, reductions) is
// fused into the epilogue of the pass that produces its inputs.
//
// Vectors live in device order (rows and columns sorted by length, see
// layout.h).  All scalars are computed redundantly by every thread of the
// team from the same reduction results, so the team stays in lockstep.
#pragma once
#include <cmath>
#include <cstdint>

#include "device.cuh"

namespace acd {

// One log record; the host formats them after the solve with the
// reference's line formats (approx.c:504-515, alm.c:260-285).
struct LogRec {
        int kind;        // 0 inner line, 1 outer line
        int restarts;    // inner: restarts since the previous inner line
        int stalled;     // outer: inner solve did not reach max_pg
        int has_delta;   // inner: delta column present
        long long k;
        double a[6];
};

struct LogBuf {
        LogRec * rec;
        int cap;
        int * count;     // records written (may exceed cap: then dropped)
};

template <class T>
struct InnerProblem {
        int m, n;
        SellDev<T> A, At;
        const T * b;
        const T * w;
        const T * c;
        const T * l;
        const T * u;
        const T * v;
        const T * inv_v;
};

// Violation vectors (m entries, w (A x - b) at some x) are stored in
// interleaved pairs: entry i of a pair's first vector at [2 i], of its
// second at [2 i + 1].  z's violation and y's always share a pair (z first),
// because the A pass that computes zp's violation also computes the next
// y's and writes both halves of zp's pair; the A' pass of the two-gradient
// step then fetches both right-hand sides of column j with one 16-byte
// (8-byte in FP32) gather instead of two.  x's violation and its
// speculative successor share the third pair.  A vector's pointer is the
// address of its entry 0; entry i is at [kViolStride * i].
constexpr int kViolStride = 2;

template <class T>
struct InnerWork {
        T * zx, * zpx, * xx, * g, * g2, * prev, * prev_alt, * alt_x, * ux;  // n
        T * vz, * vzp, * vx;  // violation pairs, 2m each: (z, y), (zp, -), (x, -)
        T * alt_xv;           // x's spare half (set by Approx::solve)
};

struct InnerArgs {
        long long niter;
        double max_pg, max_value, min_delta, offset;
        long long period;
        int log;         // record log lines
        unsigned long long t_start_ns;  // globaltimer at the solve's start
        unsigned long long limit_ns;    // give up (ACDALM_ETIMELIMIT) after this
        // When the iterate is a correction d to a point xbar (the mixed
        // precision mode), |xbar + d| is the norm the min_delta test uses.
        const double * xbar;
};

template <class T>
struct Vec {
        T * x;
        T * viol;
        int violp;
        double quad, value;  // NaN = not cached
};

template <class T>
__device__ __forceinline__ void vswap(Vec<T> & a, Vec<T> & b)
{
        Vec<T> t = a;
        a = b;
        b = t;
}

// maxpd / minpd lane rules of the reference's SSE2 code: the second operand
// wins ties and NaN.
template <class T>
__device__ __forceinline__ T maxpd(T a, T b) { return (a > b) ? a : b; }
template <class T>
__device__ __forceinline__ T minpd(T a, T b) { return (a < b) ? a : b; }

template <bool Exact>
__device__ __forceinline__ double mul(double a, double b)
{
        return Exact ? __dmul_rn(a, b) : a * b;
}
template <bool Exact>
__device__ __forceinline__ float mul(float a, float b)
{
        return Exact ? __fmul_rn(a, b) : a * b;
}
// z - g*s
template <bool Exact>
__device__ __forceinline__ double msub(double z, double g, double s)
{
        return Exact ? __dsub_rn(z, __dmul_rn(g, s)) : fma(-g, s, z);
}
template <bool Exact>
__device__ __forceinline__ float msub(float z, float g, float s)
{
        return Exact ? __fsub_rn(z, __fmul_rn(g, s)) : fmaf(-g, s, z);
}
// a*x + b*y
template <bool Exact>
__device__ __forceinline__ double lerp2(double a, double x, double b, double y)
{
        return Exact ? __dadd_rn(__dmul_rn(a, x), __dmul_rn(b, y))
                     : fma(a, x, b * y);
}
template <bool Exact>
__device__ __forceinline__ float lerp2(float a, float x, float b, float y)
{
        return Exact ? __fadd_rn(__fmul_rn(a, x), __fmul_rn(b, y))
                     : fmaf(a, x, b * y);
}

__device__ __forceinline__ bool is_nan(double v) { return v != v; }

// Reduction partials of an inner solve: FP64 for the FP64 solve, float-float
// for the FP32 one (its FP64 pipe work would otherwise bound the iteration).
template <class T>
struct AccOf {
        typedef double type;
};
template <>
struct AccOf<float> {
        typedef DF type;
};

// NaN test on the bits (integer pipe).
__device__ __forceinline__ bool nan_bits(double v)
{
        return (__double_as_longlong(v) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

template <class T, class Team, bool Exact>
struct Approx {
        typedef typename AccOf<T>::type Acc;
        Team & tm;
        InnerProblem<T> P;
        InnerWork<T> W;
        LogBuf log;
        Vec<T> y, z, zp, x;
        long long iteration;
        // momentum and step length: in T (the FP32 solve only ever uses them
        // rounded to float)
        T theta, step_length;
        int restarts_since_log;
        bool ok;
        unsigned long long t_start_ns;
        const double * xbar = nullptr;

        __device__ Approx(Team & t, const InnerProblem<T> & p,
                          const InnerWork<T> & w, const LogBuf & lb)
                : tm(t), P(p), W(w), log(lb)
        {
                ok = true;
        }

        __device__ int lane() const { return threadIdx.x & 31; }

        template <int K>
        __device__ bool reduce(const Acc (&part)[K], const int (&op)[K], double (&res)[K])
        {
                return tm.template reduce_to<K, Acc>(part, op, res);
        }

        __device__ void put_log(const LogRec & r)
        {
                if (tm.tid() == 0) {
                        int at = atomicAdd(log.count, 1);
                        if (at < log.cap)
                                log.rec[at] = r;
                }
        }

        // ---- phase: row sums of A at v.x (compute_violation) ----
        //
        // gradient_value.inc:15-81: viol = w (A x - b), quad = 1/2 sum w
        // (Ax-b)^2.  linterp: 0 none; 1 = vector.inc:249-335 applied to X and
        // Y with zp = v (x = (1-th) x + th v, x_viol likewise, y_viol =
        // (1-nth) x_viol + nth v_viol); 2 = the same into the spare buffers
        // (the caller keeps them only if the line search accepts).  Optional
        // n-vector partials of v.x: c'v (value), |v|^2 and |prev - v|^2.
        __device__ bool violation(Vec<T> & v, int linterp, T th, T nth,
                                  bool want_cx, bool want_delta, double * cx,
                                  double * xx, double * dd2, double * elapsed = nullptr)
        {
                Acc part[5] = {};
                const int op[5] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_MAX};
                const T ts = T(1) - th, tt = th, ns = T(1) - nth, nt = nth;
                constexpr int S = kViolStride;
                // with the momentum update, v is zp: the next y's violation
                // goes to the second half of v's pair, beside v's own, in
                // one pair-sized store (v.viol must start a pair)
                if (linterp &&
                    (reinterpret_cast<uintptr_t>(v.viol) & (S * sizeof(T) - 1)) != 0) {
                        tm.fail(kStatusInternal);
                        return false;
                }
                T * xvw = (linterp == 2) ? W.alt_xv : x.viol;
                T * xxw = (linterp == 2) ? W.alt_x : x.x;
                const T * xvr = x.viol;
                const T * xxr = x.x;
                struct RowPre {
                        T b, w, xv;
                };
                auto pre = [&](int i) {
                        RowPre q = {T(0), T(0), T(0)};
                        if (i >= 0) {
                                q.b = tm.ld(P.b + i);
                                q.w = tm.ld(P.w + i);
                                if (linterp)
                                        q.xv = tm.ld(xvr + S * i);
                        }
                        return q;
                };
                sell_rows_1p<Exact, 1>(tm, P.A, v.x, pre, [&](int i, T ax, const RowPre & q) {
                        T r = ax - q.b;
                        T s = mul<Exact>(q.w, r);
                        acc_prod(part[0], s, r);
                        if (linterp) {
                                T xv = lerp2<Exact>(ts, q.xv, tt, s);
                                T yv = lerp2<Exact>(ns, xv, nt, s);
                                store_pair(v.viol + S * i, s, yv);
                                xvw[S * i] = xv;
                        } else {
                                v.viol[S * i] = s;
                        }
                });
                if (linterp || want_cx || want_delta) {
                        for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                                T vj = tm.ld(v.x + j);
                                if (linterp)
                                        xxw[j] = lerp2<Exact>(ts, tm.ld(xxr + j), tt, vj);
                                if (want_cx)
                                        acc_prod(part[1], tm.ld(P.c + j), vj);
                                if (want_delta) {
                                        double d = (double)tm.ld(W.prev + j) - (double)vj;
                                        double full = xbar ? xbar[j] + (double)vj : (double)vj;
                                        acc_add(part[2], full * full);
                                        acc_add(part[3], d * d);
                                }
                        }
                }
                if (elapsed)
                        acc_max(part[4], (T)(global_ns() - t_start_ns));
                double res[5];
                if (!reduce(part, op, res))
                        return false;
                v.quad = .5 * res[0];
                v.violp = 1;
                if (elapsed)
                        *elapsed = res[4];
                if (cx)
                        *cx = res[1];
                if (xx)
                        *xx = res[2];
                if (dd2)
                        *dd2 = res[3];
                return true;
        }

        // ---- phase: A' pass + prox step (gradient2_step / gradient(2)_long_step) ----
        //
        // step_project.inc:179-312 (two, long), :320-444 (one, long),
        // :452-581 (two, short): g = A' z_viol + c (if two), g2 = A' y_viol +
        // c, zp = P[l,u](z - g2 itheta inv_v).  Partials: max |zp| (short)
        // or the long step's estimate sum g2 (zp-z) + 1/2 sum (zp-z)^2
        // theta2 v; |z - P(z - g)|^2 (pg); g (zp - z) (dot_diff); c'z; c'zp.
        struct StepOut {
                double maxz, est, pg2, dd, cz, czp;
        };
        __device__ bool at_step(bool two, bool is_long, T itheta, T theta2,
                                bool want_pg, bool want_dd, bool want_cz,
                                StepOut & o)
        {
                Acc part[6] = {};
                const int op[6] = {is_long ? RED_SUM : RED_MAX, RED_SUM, RED_SUM,
                                   RED_SUM, RED_SUM, RED_SUM};
                const T it = itheta, t2 = theta2;
                T * g = W.g;
                T * g2 = W.g2;
                struct ColPre {
                        T c, z, l, u, iv, v;
                };
                auto pre = [&](int j) {
                        ColPre q = {T(0), T(0), T(0), T(0), T(0), T(0)};
                        if (j >= 0) {
                                q.c = tm.ld(P.c + j);
                                q.z = tm.ld(z.x + j);
                                q.l = tm.ld(P.l + j);
                                q.u = tm.ld(P.u + j);
                                q.iv = tm.ld(P.inv_v + j);
                                if (is_long)
                                        q.v = tm.ld(P.v + j);
                        }
                        return q;
                };
                auto epi = [&](int j, T g0, T g1, const ColPre & q) {
                        T cj = q.c;
                        if (two)
                                g0 = g0 + cj;
                        g1 = g1 + cj;
                        if (two)
                                g[j] = g0;
                        g2[j] = g1;
                        T zj = q.z;
                        T lj = q.l, uj = q.u;
                        T stp = mul<Exact>(it, q.iv);
                        T trial = msub<Exact>(zj, g1, stp);
                        trial = maxpd(lj, trial);
                        trial = minpd(uj, trial);
                        zp.x[j] = trial;
                        T delta = trial - zj;
                        if (is_long) {
                                acc_prod(part[0], g1, delta);
                                acc_add(part[1], delta * delta * t2 * q.v);
                        } else {
                                acc_max(part[0], fabs(trial));
                        }
                        if (want_pg) {
                                T xp = zj - g0;
                                xp = maxpd(lj, xp);
                                xp = minpd(uj, xp);
                                T d = zj - xp;
                                acc_prod(part[2], d, d);
                        }
                        if (want_dd)
                                acc_prod(part[3], g0, delta);
                        if (want_cz)
                                acc_prod(part[4], cj, zj);
                        acc_prod(part[5], cj, trial);
                };
                if (two) {
                        if (y.viol != z.viol + 1) {  // the pairing invariant
                                tm.fail(kStatusInternal);
                                return false;
                        }
                        sell_rows_pair<Exact>(tm, P.At, z.viol, pre, epi);
                } else {
                        sell_rows_1p<Exact, kViolStride>(tm, P.At, y.viol, pre,
                                                         [&](int j, T g1, const ColPre & q) {
                                                                 epi(j, (T)0, g1, q);
                                                         });
                }
                double res[6];
                if (!reduce(part, op, res))
                        return false;
                o.maxz = is_long ? 0 : res[0];
                o.est = is_long ? res[0] + .5 * res[1] : 0;
                o.pg2 = res[2];
                o.dd = res[3];
                o.cz = res[4];
                o.czp = res[5];
                return true;
        }

        // ---- phase: gradient(g, v) (gradient_value.inc:142-181) ----
        // g = A' v_viol + c; partials |v - P(v - g)|^2 and |g|^2; optionally
        // copies v.x into prev_alt.
        __device__ bool gradient(const Vec<T> & v, bool copy_prev, double & pg2,
                                 double & gg)
        {
                Acc part[2] = {};
                const int op[2] = {RED_SUM, RED_SUM};
                T * g = W.g;
                sell_rows_1<Exact, kViolStride>(tm, P.At, v.viol, [&](int j, T a) {
                        T gj = a + tm.ld(P.c + j);
                        g[j] = gj;
                        T xj = tm.ld(v.x + j);
                        T xp = xj - gj;
                        xp = maxpd(tm.ld(P.l + j), xp);
                        xp = minpd(tm.ld(P.u + j), xp);
                        T d = xj - xp;
                        acc_prod(part[0], d, d);
                        acc_prod(part[1], gj, gj);
                        if (copy_prev)
                                W.prev_alt[j] = xj;
                });
                double res[2];
                if (!reduce(part, op, res))
                        return false;
                pg2 = res[0];
                gg = res[1];
                return true;
        }

        // ---- phase: the retry after a rejected unsafe long step ----
        // step_project.inc:34-94 (zp = P(z - g2 (1-1e-6)/theta inv_v)),
        // preceded, when the pass did not produce it, by gradient(g, z); and
        // dot_diff (approx.c:227-256) on the new zp.
        __device__ bool retry_step(bool need_grad, double & dd)
        {
                Acc part[1] = {};
                const int op[1] = {RED_SUM};
                const T it = T(1 - 1e-6) / theta;
                T * g = W.g;
                auto body = [&](int j, T gj) {
                        T zj = tm.ld(z.x + j);
                        T stp = mul<Exact>(it, tm.ld(P.inv_v + j));
                        T trial = msub<Exact>(zj, tm.ld(W.g2 + j), stp);
                        trial = maxpd(tm.ld(P.l + j), trial);
                        trial = minpd(tm.ld(P.u + j), trial);
                        zp.x[j] = trial;
                        acc_prod(part[0], gj, trial - zj);
                };
                if (need_grad) {
                        sell_rows_1<Exact, kViolStride>(tm, P.At, z.viol, [&](int j, T a) {
                                T gj = a + tm.ld(P.c + j);
                                g[j] = gj;
                                body(j, gj);
                        });
                } else {
                        for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                                body(j, tm.ld(g + j));
                }
                double res[1];
                if (!reduce(part, op, res))
                        return false;
                dd = res[0];
                return true;
        }

        // ---- phase: restart copies x <- z, y <- z (approx.c:449-457) ----
        __device__ bool restart_copy()
        {
                for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                        x.x[j] = tm.ld(z.x + j);
                for (int i = tm.tid(); i < P.m; i += tm.nthreads()) {
                        T zi = tm.ld(z.viol + kViolStride * i);
                        x.viol[kViolStride * i] = zi;
                        y.viol[kViolStride * i] = zi;
                }
                x.violp = y.violp = z.violp;
                x.quad = y.quad = z.quad;
                x.value = y.value = z.value;
                return tm.sync();
        }

        // c' v when v.value is not cached; computes the violation if needed
        // (gradient_value.inc:111-133).
        __device__ bool value_of(Vec<T> & v, double & out)
        {
                if (!nan_bits(v.value)) {
                        out = v.value;
                        return true;
                }
                double cx = 0;
                if (nan_bits(v.quad) || !v.violp) {
                        if (!violation(v, 0, 0, 0, true, false, &cx, nullptr, nullptr))
                                return false;
                } else {
                        Acc part[1] = {};
                        const int op[1] = {RED_SUM};
                        for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                                acc_prod(part[0], tm.ld(P.c + j), tm.ld(v.x + j));
                        double res[1];
                        if (!reduce(part, op, res))
                                return false;
                        cx = res[0];
                }
                v.value = v.quad + cx;
                out = v.value;
                return true;
        }

        __device__ bool norms_vs_prev(const Vec<T> & v, double & xx, double & dd2)
        {
                Acc part[2] = {};
                const int op[2] = {RED_SUM, RED_SUM};
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        double vj = (double)tm.ld(v.x + j);
                        double d = (double)tm.ld(W.prev + j) - vj;
                        double full = xbar ? xbar[j] + vj : vj;
                        acc_add(part[0], full * full);
                        acc_add(part[1], d * d);
                }
                double res[2];
                if (!reduce(part, op, res))
                        return false;
                xx = res[0];
                dd2 = res[1];
                return true;
        }

        __device__ bool norm_g(double & gg)
        {
                Acc part[1] = {};
                const int op[1] = {RED_SUM};
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        T gj = tm.ld(W.g + j);
                        acc_prod(part[0], gj, gj);
                }
                double res[1];
                if (!reduce(part, op, res))
                        return false;
                gg = res[0];
                return true;
        }

        __device__ static void invalidate(Vec<T> & v)
        {
                v.violp = 0;
                v.quad = v.value = NAN;
        }

        __device__ bool check_finite(double maxz)
        {
                if (!(maxz < HUGE_VAL)) {  // step_project.inc:90, :577
                        tm.fail(kStatusNonFinite);
                        return false;
                }
                return true;
        }

        // One APPROX iteration (approx.c:417-478).  Returns 0 when the
        // center is the zp slot (the previous z) and 1 after a restart
        // (center = x); -1 on failure.
        __device__ int iter(bool want_pg, double & out_pg)
        {
                bool descent, got_gradient;
                T stepl = step_length;
                double dd = 0;
                bool dd_valid = false;
                bool spec_valid = false;  // alt buffers hold linterp of zp
                T th = theta;
                T nth = T(2) / ((T)(iteration + 1) + T(2));
                if (stepl <= 1) {
                        // short_step, approx.c:394-415
                        StepOut o;
                        bool want_cz = nan_bits(z.value);
                        if (!at_step(true, false, T(1 - 1e-6) / th, T(0), want_pg, true,
                                     want_cz, o))
                                return -1;
                        if (!check_finite(o.maxz))
                                return -1;
                        if (want_cz)
                                z.value = z.quad + o.cz;
                        invalidate(zp);
                        step_length = stepl * T(1.01);
                        if (step_length > T(1))
                                step_length = T(1 + 1e-6);
                        descent = false;
                        got_gradient = true;
                        dd = o.dd;
                        dd_valid = true;
                        if (want_pg)
                                out_pg = sqrt(o.pg2);
                } else {
                        // try_long_step, approx.c:343-392
                        got_gradient = want_pg || (stepl <= T(1 + 1e-6));
                        bool safe = (stepl <= T(1 + 1e-6));
                        T len = safe ? T(1) : stepl;
                        StepOut o;
                        bool want_cz = nan_bits(z.value);
                        if (!at_step(got_gradient, true, (len - T(1e-6)) / th, th / len,
                                     want_pg, got_gradient, want_cz, o))
                                return -1;
                        if (want_cz)
                                z.value = z.quad + o.cz;
                        invalidate(zp);
                        double initial = z.value;
                        // compute_value(zp): A pass on zp, with the momentum
                        // update prepared in the spare buffers.
                        if (!violation(zp, 2, th, nth, false, false, nullptr, nullptr,
                                       nullptr))
                                return -1;
                        zp.value = zp.quad + o.czp;
                        double now = zp.value;
                        spec_valid = true;
                        if (want_pg)
                                out_pg = sqrt(o.pg2);
                        if (got_gradient) {
                                dd = o.dd;
                                dd_valid = true;
                        }
                        if (now <= initial + o.est) {
                                step_length = len * T(1.01);
                                descent = true;
                        } else {
                                step_length = T(.9) * len;
                                descent = false;
                                if (!safe) {
                                        if (!retry_step(!got_gradient, dd))
                                                return -1;
                                        dd_valid = true;
                                        invalidate(zp);
                                        spec_valid = false;
                                }
                        }
                }
                if (!descent) {
                        if (!dd_valid) {  // unreachable: kept for safety
                                tm.fail(kStatusInternal);
                                return -1;
                        }
                        if (dd > 0) {
                                // oscillation: restart, approx.c:449-457
                                if (!restart_copy())
                                        return -1;
                                iteration = 0;
                                theta = 1;
                                return 1;
                        }
                }
                if (spec_valid && zp.violp) {
                        // adopt the momentum update computed speculatively
                        T * t = x.viol; x.viol = W.alt_xv; W.alt_xv = t;
                        t = x.x; x.x = W.alt_x; W.alt_x = t;
                } else {
                        if (!violation(zp, 1, th, nth, false, false, nullptr, nullptr,
                                       nullptr))
                                return -1;
                }
                // the next y's violation is the second half of zp's pair
                y.viol = zp.viol + 1;
                iteration += 1;
                theta = nth;
                y.value = x.value = NAN;
                y.quad = x.quad = NAN;
                vswap(z, zp);
                return 0;
        }

        // approx_solve, approx.c:576-708, from x_io (device order, projected
        // here); the center is copied back to x_io.  Returns the reason
        // (0..3) or -1 on failure; diag = value, |g|, |pg|, delta, iterations.
        __device__ int solve(const InnerArgs & a, T * x_io, double * diag,
                             long long * iters_out)
        {
                t_start_ns = a.t_start_ns;
                xbar = a.xbar;
                // state init (approx.c:588-603)
                y = {nullptr, W.vz + 1, 0, NAN, NAN};
                z = {W.zx, W.vz, 0, NAN, NAN};
                zp = {W.zpx, W.vzp, 0, NAN, NAN};
                x = {W.xx, W.vx, 0, NAN, NAN};
                W.alt_xv = W.vx + 1;
                iteration = 0;
                theta = 1;
                step_length = 1;
                restarts_since_log = 0;
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        T xj = tm.ld(x_io + j);
                        T lo = maxpd(tm.ld(P.l + j), xj);
                        x.x[j] = minpd(lo, tm.ld(P.u + j));
                }
                if (!tm.sync())
                        return -1;
                double cx;
                if (!violation(x, 0, 0, 0, true, false, &cx, nullptr, nullptr))
                        return -1;
                x.value = x.quad + cx;
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        T v = tm.ld(x.x + j);
                        z.x[j] = v;
                        W.prev[j] = v;
                }
                for (int i = tm.tid(); i < P.m; i += tm.nthreads()) {
                        T v = tm.ld(x.viol + kViolStride * i);
                        store_pair(z.viol + kViolStride * i, v, v);  // z and y
                }
                z.violp = y.violp = 1;
                z.quad = y.quad = x.quad;
                z.value = y.value = x.value;
                if (!tm.sync())
                        return -1;

                int center = 1;  // 1 = x, 0 = zp slot
                double value = x.value + a.offset;
                double ng = HUGE_VAL, pg = HUGE_VAL, delta = HUGE_VAL;
                long long i;
                int reason = 0;
                for (i = 0; i < a.niter; i++) {
                        delta = HUGE_VAL;
                        pg = HUGE_VAL;
                        bool want_pg = (i == 0) || ((i + 1) % 10 == 0);
                        center = iter(want_pg, pg);
                        if (center < 0)
                                return -1;
                        if (center == 1)
                                restarts_since_log++;
                        Vec<T> & cv = center ? x : zp;
                        double cval;
                        if (!value_of(cv, cval))
                                return -1;
                        value = cval + a.offset;
                        if (value < a.max_value) {
                                reason = 1;
                                break;
                        }
                        if (pg < a.max_pg) {
                                reason = 2;
                                break;
                        }
                        if ((i + 1) % 100 == 0) {
                                center = 1;
                                                double cxx, xx, dd2, elapsed;
                                if (!violation(x, 0, 0, 0, true, true, &cxx, &xx, &dd2,
                                               &elapsed))
                                        return -1;
                                // bounded runtime: every thread sees the same
                                // (reduced) elapsed time, so all stop together
                                if (a.limit_ns && elapsed > (double)a.limit_ns) {
                                        tm.fail(kStatusTimeLimit);
                                        return -1;
                                }
                                if (is_nan(x.value))
                                        x.value = x.quad + cxx;
                                value = x.value + a.offset;
                                double pg2, gg;
                                if (!gradient(x, true, pg2, gg))
                                        return -1;
                                pg = sqrt(pg2);
                                delta = sqrt(dd2) / (sqrt(xx) + 1e-10);
                                if (value < a.max_value) {
                                        reason = 1;
                                        break;
                                }
                                if (pg < a.max_pg) {
                                        reason = 2;
                                        break;
                                }
                                if (delta < a.min_delta) {
                                        reason = 3;
                                        break;
                                }
                                T * t = W.prev; W.prev = W.prev_alt; W.prev_alt = t;
                        }
                        if (a.log && ((i == 0) || (a.period && ((i + 1) % a.period == 0)))) {
                                double gg;
                                if (!norm_g(gg))
                                        return -1;
                                ng = sqrt(gg);
                                LogRec r = {0, restarts_since_log, 0, delta < HUGE_VAL,
                                            i + 1, {value, ng, pg, step_length, delta, 0}};
                                put_log(r);
                                restarts_since_log = 0;
                        }
                }
                // exit diagnostics, approx.c:681-702
                Vec<T> & cv = center ? x : zp;
                double xx, dd2;
                if (!norms_vs_prev(cv, xx, dd2))
                        return -1;
                delta = sqrt(dd2) / (sqrt(xx) + 1e-10);
                double cval;
                if (!value_of(cv, cval))
                        return -1;
                value = cval + a.offset;
                if (!cv.violp) {
                        double dummy;
                        if (!violation(cv, 0, 0, 0, false, false, &dummy, nullptr, nullptr))
                                return -1;
                }
                double pg2, gg;
                if (!gradient(cv, false, pg2, gg))
                        return -1;
                ng = sqrt(gg);
                pg = sqrt(pg2);
                if (a.log) {
                        LogRec r = {0, restarts_since_log, 0, delta < HUGE_VAL, i + 1,
                                    {value, ng, pg, step_length, delta, 0}};
                        put_log(r);
                }
                for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                        x_io[j] = tm.ld(cv.x + j);
                if (!tm.sync())
                        return -1;
                diag[0] = value;
                diag[1] = ng;
                diag[2] = pg;
                diag[3] = delta;
                diag[4] = (double)(i + 1);
                *iters_out = (reason == 0) ? i : i + 1;
                return reason;
        }
};


// ---------------------------------------------------------------------
// ALM outer loop (alm.c:106-322), FP64 throughout.
// ---------------------------------------------------------------------

struct AlmProblem {
        int m, n;
        SellDev<double> A, At;
        const double * b;        // m
        const double * c0;       // n, the LP objective
        const double * l;        // n
        const double * u;        // n
        const double * lam_lo;   // m
        const double * lam_hi;   // m
        const double * beta;     // m, nonzeros per row
        const int32_t * orig_row;// m, original row of each device row
        double * w;              // m, ALM weights (persist across solves)
        double * c;              // n, c0 - A' lambda (the inner linear term)
        double * v;              // n, ESO step constants
        double * inv_v;          // n
        double * r;              // m, A x - b
        double bnorm, cnorm;     // |b|_2, |c0|_2 (for the relative KKT)
};

struct AlmArgs {
        long long niter;
        unsigned long long inner_budget;  // 0 = none
        double kkt_tol;                   // 0 = off
        int log;
        unsigned long long limit_ns;      // whole-solve time limit (0 = none)
        // mixed precision (FP32 inner iterations on the correction to an
        // FP64 point, FP64 everywhere else)
        int mixed;
        double min_delta32;               // the FP32 inner solves' stall test
        long long niter32;                // cap per FP32 inner solve
        double pg_floor32;                // FP32 projected-gradient floor / |c'|
        int stall_switch;                 // FP32 stalls in a row before the
                                          // remaining outer iterations run FP64
};

// The FP32 copies the mixed mode works on (device order).
struct AlmMixed {
        SellDev<float> Af, Atf;
        float * bf, * wf;                              // m
        float * cf, * lf, * uf, * vf, * ivf, * d;      // n
        InnerWork<float> Wf;
};

struct AlmOut {
        int ret;                 // 0 almost feasible, 1 iteration limit
        double diag[3];          // objective, max violation, pg
        long long outer;
        unsigned long long inner;
        unsigned long long inner32;  // of which FP32 (mixed mode)
        double primal, dual, gap, rel_kkt, objective;
};

template <class Team, bool Exact>
struct Alm {
        Team & tm;
        AlmProblem P;
        InnerWork<double> W;
        LogBuf log;
        AlmMixed mixed;

        __device__ Alm(Team & t, const AlmProblem & p, const InnerWork<double> & w,
                       const LogBuf & lb, const AlmMixed & mxd)
                : tm(t), P(p), W(w), log(lb), mixed(mxd) {}

        // penalise_linear (alm.c:106-119) + approx_update_step_size of the
        // permuted instance (approx.c:135-186) in one pass over A':
        // c = c0 - A' lambda; v_j = sum_i w_i beta_i A_ij^2 in the
        // reference's order and rounding (bit-identical); inv_v = 1/v (1
        // where v = 0 and c = 0).  Partials: lambda'b, and the relative KKT
        // terms of (x, lambda) when kkt is set.
        __device__ bool penalise(const double * lam, const double * x, bool kkt,
                                 double (&out)[7], bool write = true,
                                 const AlmMixed * mx = nullptr)
        {
                double part[7] = {0, 0, 0, 0, 0, 0, 0};
                const int op[7] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_SUM, RED_SUM};
                int lane = threadIdx.x & 31;
                const SellDev<double> & op_t = P.At;
                for_each_slice(tm, op_t.nslices, [&](int s) {
                        Slice sl = slice_of(op_t, s, lane);
                        double acc = 0, vv = 0;
                        by_width(sl, [&](auto wv) {
                                constexpr int VEC = decltype(wv)::value;
                                int64_t at = sl.base + VEC * lane;
                                for (int k = 0; k < sl.steps; k++, at += 32 * VEC) {
                                        Chunk<VEC, double> q =
                                                load_chunk<VEC>(op_t.col, op_t.val, at);
                                        double t[VEC], pl[VEC];
#pragma unroll
                                        for (int j = 0; j < VEC; j++) {
                                                int i = q.c[j];
                                                // v in the reference's order and rounding
                                                t[j] = __dmul_rn(__dmul_rn(__dmul_rn(tm.ld(P.w + i),
                                                                                     P.beta[i]),
                                                                           q.a[j]),
                                                                 q.a[j]);
                                                pl[j] = tm.ld(lam + i);
                                        }
                                        vv = in_order<VEC>(vv, t, sl.shift, lane);
                                        if constexpr (Exact) {
#pragma unroll
                                                for (int j = 0; j < VEC; j++)
                                                        pl[j] = __dmul_rn(q.a[j], pl[j]);
                                                acc = in_order<VEC>(acc, pl, sl.shift, lane);
                                        } else {
#pragma unroll
                                                for (int j = 0; j < VEC; j++)
                                                        acc = fma(q.a[j], pl[j], acc);
                                        }
                                }
                                if constexpr (!Exact)
                                        acc = finish_row(acc, sl.shift, (sl.steps * VEC) << sl.shift);
                                return 0;
                        });
                        int j = sl.row;
                        if (sl.lead && j < P.n) {
                                double cj = P.c0[j] - acc;
                                if (write) {
                                        double ivj = (vv == 0 && cj == 0) ? 1.0 : 1.0 / vv;
                                        P.c[j] = cj;
                                        P.v[j] = vv;
                                        P.inv_v[j] = ivj;
                                        if (mx) {
                                                // the FP32 inner problem in the
                                                // correction d = x - xbar
                                                double xj = tm.ld(x + j);
                                                mx->cf[j] = (float)cj;
                                                mx->vf[j] = (float)vv;
                                                mx->ivf[j] = (float)ivj;
                                                mx->lf[j] = (float)(P.l[j] - xj);
                                                mx->uf[j] = (float)(P.u[j] - xj);
                                                mx->d[j] = 0.f;
                                                part[5] += cj * xj;
                                                part[6] += cj * cj;
                                        }
                                }
                                if (kkt) {
                                        double xj = tm.ld(x + j);
                                        double xp = xj - cj;
                                        xp = fmax(P.l[j], fmin(xp, P.u[j]));
                                        double d = xj - xp;
                                        part[1] += d * d;
                                        part[2] += P.c0[j] * xj;
                                        double lo = isfinite(P.l[j]) ? P.l[j] * cj : HUGE_VAL;
                                        double hi = isfinite(P.u[j]) ? P.u[j] * cj : HUGE_VAL;
                                        double t = fmin(lo, hi);
                                        part[3] += isfinite(t) ? t : 0.0;
                                }
                        }
                });
                for (int i = tm.tid(); i < P.m; i += tm.nthreads()) {
                        double li = tm.ld(lam + i);
                        part[0] += li * P.b[i];
                        if (kkt) {
                                double ri = tm.ld(P.r + i);
                                part[4] += ri * ri;
                        }
                        if (mx && write) {
                                mx->bf[i] = (float)(-tm.ld(P.r + i));
                                mx->wf[i] = (float)tm.ld(P.w + i);
                        }
                }
                if (!tm.reduce(part, op))
                        return false;
                for (int k = 0; k < 7; k++)
                        out[k] = part[k];
                return true;
        }

        // violation (alm.c:121-132) fused with update_multipliers
        // (alm.c:182-192): r = A x - b, lambda = P[lo,hi](lambda - w r).
        // Partials: max |r|, |r|^2, |w|_1, c0'x.
        __device__ bool violation(const double * x, double * lam, double (&out)[4])
        {
                double part[4] = {-HUGE_VAL, 0, 0, 0};
                const int op[4] = {RED_MAX, RED_SUM, RED_SUM, RED_SUM};
                sell_rows_1<Exact>(tm, P.A, x, [&](int i, double ax) {
                        double ri = ax - P.b[i];
                        P.r[i] = ri;
                        double a = fabs(ri);
                        part[0] = (a > part[0]) ? a : part[0];
                        part[1] += ri * ri;
                        double wi = tm.ld(P.w + i);
                        part[2] += fabs(wi);
                        double li = tm.ld(lam + i) - wi * ri;
                        lam[i] = fmax(P.lam_lo[i], fmin(li, P.lam_hi[i]));
                });
                for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                        part[3] += P.c0[j] * tm.ld(x + j);
                if (!tm.reduce(part, op))
                        return false;
                for (int k = 0; k < 4; k++)
                        out[k] = part[k];
                return true;
        }

        // First original row index among the rows with |r| == maxr
        // (norm_inf's tie rule, alm.c:154-169).
        __device__ bool argmax_row(double maxr, int & d_out)
        {
                double part[2] = {HUGE_VAL, HUGE_VAL};
                const int op[2] = {RED_MIN, RED_MIN};
                for (int i = tm.tid(); i < P.m; i += tm.nthreads()) {
                        if (fabs(tm.ld(P.r + i)) == maxr) {
                                double o = (double)P.orig_row[i];
                                if (o < part[0]) {
                                        part[0] = o;
                                        part[1] = (double)i;
                                }
                        }
                }
                // the device row of the smallest original row: a second
                // pass keyed on it keeps the pair consistent
                if (!tm.reduce(part, op))
                        return false;
                double best = part[0];
                double q[1] = {HUGE_VAL};
                const int op1[1] = {RED_MIN};
                for (int i = tm.tid(); i < P.m; i += tm.nthreads())
                        if ((double)P.orig_row[i] == best && fabs(tm.ld(P.r + i)) == maxr)
                                q[0] = (double)i;
                if (!tm.reduce(q, op1))
                        return false;
                d_out = (int)q[0];
                return true;
        }

        // update_weights (alm.c:194-212) after the argmax; returns |w|_1.
        __device__ bool scale_weights(double scale, int bump_row, double & wsum)
        {
                double part[1] = {0};
                const int op[1] = {RED_SUM};
                for (int i = tm.tid(); i < P.m; i += tm.nthreads()) {
                        double wi = tm.ld(P.w + i) * scale;
                        if (i == bump_row)
                                wi *= 10;
                        P.w[i] = wi;
                        part[0] += fabs(wi);
                }
                if (!tm.reduce(part, op))
                        return false;
                wsum = part[0];
                return true;
        }

        __device__ void put_log(const LogRec & r)
        {
                if (tm.tid() == 0) {
                        int at = atomicAdd(log.count, 1);
                        if (at < log.cap)
                                log.rec[at] = r;
                }
        }

        // r = A x - b (FP64), without touching the multipliers.
        __device__ bool residual(const double * x)
        {
                sell_rows_1<Exact>(tm, P.A, x, [&](int i, double ax) { P.r[i] = ax - P.b[i]; });
                return tm.sync();
        }

        // x <- P[l,u](x + d) in FP64 after an FP32 inner solve on d.
        __device__ bool apply_correction(double * x, const float * d)
        {
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        double v = tm.ld(x + j) + (double)tm.ld(d + j);
                        x[j] = fmax(P.l[j], fmin(v, P.u[j]));
                }
                return tm.sync();
        }

        // alm_solve, alm.c:289-322; x (n) and lam (m) in device order.
        __device__ int solve(const AlmArgs & a, double * x, double * lam, AlmOut & out)
        {
                unsigned long long t_start = global_ns();
                for (int i = tm.tid(); i < P.m; i += tm.nthreads())
                        lam[i] = fmax(P.lam_lo[i], fmin(tm.ld(lam + i), P.lam_hi[i]));
                if (!tm.sync())
                        return -1;
                double prev_viol_norm = HUGE_VAL, precision = 1;
                double pg = HUGE_VAL, max_viol = HUGE_VAL, cx = 0, rnorm2 = 0;
                unsigned long long inner_used = 0;
                int ret = 1;
                long long k;
                bool kkt = a.kkt_tol > 0;
                double kk[7];
                InnerProblem<double> ip;
                ip.m = P.m;
                ip.n = P.n;
                ip.A = P.A;
                ip.At = P.At;
                ip.b = P.b;
                ip.w = P.w;
                ip.c = P.c;
                ip.l = P.l;
                ip.u = P.u;
                ip.v = P.v;
                ip.inv_v = P.inv_v;
                const AlmMixed * mx = a.mixed ? &mixed : nullptr;
                bool fp64_inner = false;
                bool last_was_fp32 = false;
                double best_rk = HUGE_VAL;
                int stalls = 0;
                unsigned long long inner32 = 0;
                InnerProblem<float> ipf;
                if (mx) {
                        ipf.m = P.m;
                        ipf.n = P.n;
                        ipf.A = mixed.Af;
                        ipf.At = mixed.Atf;
                        ipf.b = mixed.bf;
                        ipf.w = mixed.wf;
                        ipf.c = mixed.cf;
                        ipf.l = mixed.lf;
                        ipf.u = mixed.uf;
                        ipf.v = mixed.vf;
                        ipf.inv_v = mixed.ivf;
                        if (!residual(x))
                                return -1;
                }
                for (k = 0; k < a.niter; k++) {
                        if (!penalise(lam, x, kkt && k > 0, kk, true,
                                      (mx && !fp64_inner) ? mx : nullptr))
                                return -1;
                        if (kkt && k > 0) {
                                double primal = sqrt(kk[4]) / (1 + P.bnorm);
                                double dual = sqrt(kk[1]) / (1 + P.cnorm);
                                double dobj = kk[0] + kk[3];
                                double gap = fabs(kk[2] - dobj) / (1 + fabs(kk[2]) + fabs(dobj));
                                double rk = fmax(primal, fmax(dual, gap));
                                out.primal = primal;
                                out.dual = dual;
                                out.gap = gap;
                                out.rel_kkt = rk;
                                if (rk <= a.kkt_tol) {
                                        ret = 0;
                                        break;
                                }
                                // mixed mode: FP32 inner solves that stop
                                // improving the KKT residual hand over to FP64
                                // (the final outer iterations refine in FP64)
                                if (mx && !fp64_inner && last_was_fp32) {
                                        stalls = (rk > 0.9 * best_rk) ? stalls + 1 : 0;
                                        if (stalls >= a.stall_switch)
                                                fp64_inner = true;
                                }
                                best_rk = fmin(best_rk, rk);
                        }
                        double offset = kk[0];
                        InnerArgs ia;
                        ia.niter = 4294967295ll;  // -1u, alm.c:255
                        if (a.inner_budget) {
                                unsigned long long left = (inner_used < a.inner_budget)
                                        ? a.inner_budget - inner_used : 0;
                                if ((unsigned long long)ia.niter > left)
                                        ia.niter = (long long)left;
                        }
                        ia.max_pg = fmin(1.0, precision);
                        ia.max_value = -HUGE_VAL;
                        ia.min_delta = 1e-11;
                        ia.offset = offset;
                        ia.period = 10000;
                        ia.log = a.log;
                        ia.t_start_ns = t_start;
                        ia.limit_ns = a.limit_ns;
                        ia.xbar = nullptr;
                        double diag[5];
                        long long used = 0;
                        int reason;
                        if (mx && !fp64_inner) {
                                // FP32 iterations on the correction d to x:
                                // same problem shifted by x, so the rounding
                                // applies to d (iterative refinement)
                                InnerArgs fa = ia;
                                fa.offset = ia.offset + kk[5];
                                fa.min_delta = fmax(ia.min_delta, a.min_delta32);
                                // the projected gradient FP32 can resolve:
                                // reaching it counts as reaching max_pg
                                fa.max_pg = fmax(ia.max_pg, a.pg_floor32 * (sqrt(kk[6]) + 1));
                                if (a.niter32 > 0 && fa.niter > a.niter32)
                                        fa.niter = a.niter32;
                                fa.xbar = x;
                                Approx<float, Team, Exact> apf(tm, ipf, mx->Wf, log);
                                reason = apf.solve(fa, mx->d, diag, &used);
                                if (reason < 0)
                                        return -1;
                                inner32 += (unsigned long long)used;
                                if (!apply_correction(x, mx->d))
                                        return -1;
                                last_was_fp32 = true;
                                if (!kkt) {
                                        // no KKT residual to watch: FP32 solves
                                        // that stall hand over to FP64
                                        stalls = (reason == 2) ? 0 : stalls + 1;
                                        if (stalls >= a.stall_switch)
                                                fp64_inner = true;
                                }
                        } else {
                                Approx<double, Team, Exact> ap(tm, ip, W, log);
                                reason = ap.solve(ia, x, diag, &used);
                                if (reason < 0)
                                        return -1;
                                last_was_fp32 = false;
                        }
                        inner_used += (unsigned long long)used;
                        double vo[4];
                        if (!violation(x, lam, vo))
                                return -1;
                        max_viol = vo[0];
                        rnorm2 = vo[1];
                        double wsum = vo[2];
                        cx = vo[3];
                        double norm = sqrt(rnorm2);
                        pg = diag[2];
                        LogRec rec = {1, 0, reason != 2, 0, k + 1,
                                      {max_viol, norm, diag[2], diag[0], cx, 0}};
                        bool stalled = (reason != 2);
                        if (!stalled) {
                                if (!(norm < .5 * prev_viol_norm)) {
                                        double scale = 2 * fmin(1.0, norm / prev_viol_norm);
                                        int bump = -1;
                                        if (max_viol > .5 * norm) {
                                                if (!argmax_row(max_viol, bump))
                                                        return -1;
                                        }
                                        if (!scale_weights(scale, bump, wsum))
                                                return -1;
                                }
                                prev_viol_norm = norm;
                        }
                        // update_precision, alm.c:235-245
                        double wavg = (double)P.m / wsum;
                        precision = fmin(precision, fmin(max_viol, pow(wavg, 1.5)));
                        precision = fmax(precision, 1e-7);
                        rec.a[5] = wsum / (double)P.m;
                        if (a.log)
                                put_log(rec);
                        // the reference's stop (alm.c:306-308); a relative
                        // KKT tolerance, when set, is the stop instead
                        if (!kkt && (max_viol < 1e-5) && (stalled || pg < 1e-5)) {
                                ret = 0;
                                k++;
                                break;
                        }
                        if (a.inner_budget && inner_used >= a.inner_budget) {
                                k++;
                                break;
                        }
                }
                // final relative KKT of (x, lambda); c, v, 1/v keep the
                // last outer iteration's values (approx_linear, alm.c:109-116)
                if (!penalise(lam, x, true, kk, false))
                        return -1;
                {
                        double primal = sqrt(kk[4]) / (1 + P.bnorm);
                        double dual = sqrt(kk[1]) / (1 + P.cnorm);
                        double dobj = kk[0] + kk[3];
                        double gap = fabs(kk[2] - dobj) / (1 + fabs(kk[2]) + fabs(dobj));
                        out.primal = primal;
                        out.dual = dual;
                        out.gap = gap;
                        out.rel_kkt = fmax(primal, fmax(dual, gap));
                        out.objective = kk[2];
                }
                out.ret = ret;
                out.diag[0] = cx;
                out.diag[1] = max_viol;
                out.diag[2] = pg;
                out.outer = k;
                out.inner = inner_used;
                out.inner32 = inner32;
                return ret;
        }
};

}  // namespace acd
