// approx_t and alm_t: the reference's approx.h / alm.h API over the device
// solver.  Host mirrors keep the vectors the accessors hand out (callers may
// edit them, alm.c does too); the device copies live in a DevInstance built
// on first use from the permuted shadow matrix (approx.c:84-88).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/acdalm_ext.h"
#include "../../include/alm.h"
#include "../../include/approx.h"
#include "common.h"
#include "instance.h"
#include "layout.h"
#include "objects.h"

namespace acd {
HostMatrix & host_of(sparse_matrix_t * m);
}

namespace {

std::vector<double> copy_or(const double * src, size_t n, double missing)
{
        std::vector<double> v(n ? n : 0);
        for (size_t i = 0; i < n; i++)
                v[i] = src ? src[i] : missing;
        return v;
}

int ensure_device(approx_t * a)
{
        if (a->dev_ready)
                return 0;
        if (!acd::device_ready())
                return ACDALM_ENODEV;
        if (!a->lay_ready) {
                acd::build_device_layout(acd::host_of(a->permuted), a->lay, a->lay_max_steps);
                a->lay_ready = true;
        }
        int r = a->dev.create(a->lay);
        if (r) {
                a->dev.destroy();
                return r;
        }
        a->dev_ready = true;
        return 0;
}

// The reference asserts that its iterates stay finite
// (approx/step_project.inc:90, :577); a non-finite input makes them NaN
// from the first step, so inputs are checked here instead: no NaN
// anywhere, and infinities only in the bounds.
int check_finite(const char * who, const char * what, const double * v, size_t n,
                 bool bound)
{
        if (!v)
                return 0;
        for (size_t i = 0; i < n; i++) {
                double e = v[i];
                if (e != e || (!bound && std::isinf(e))) {
                        acd::set_error(ACDALM_ENONFINITE, "%s: %s[%zu] is %g", who, what, i, e);
                        return ACDALM_ENONFINITE;
                }
        }
        return 0;
}

int check_approx_inputs(const char * who, approx_t * a, const double * x)
{
        int r;
        if ((r = check_finite(who, "rhs", a->s_rhs.data(), a->nrhs, false))
            || (r = check_finite(who, "weight", a->s_weight.data(), a->nrhs, false))
            || (r = check_finite(who, "linear", a->s_linear.data(), a->nvars, false))
            || (r = check_finite(who, "lower", a->s_lower.data(), a->nvars, true))
            || (r = check_finite(who, "upper", a->s_upper.data(), a->nvars, true))
            || (r = check_finite(who, "x", x, a->nvars, false)))
                return r;
        return 0;
}

acd::HostVectors shadow_vectors(approx_t * a)
{
        acd::HostVectors hv;
        hv.b = a->s_rhs.data();
        hv.w = a->s_weight.data();
        hv.c0 = a->s_linear.data();
        hv.l = a->s_lower.data();
        hv.u = a->s_upper.data();
        return hv;
}

}  // namespace

extern "C" {

approx_t * approx_make(sparse_matrix_t * constraints, size_t nrhs, const double * rhs,
                       const double * weight, size_t nvars, const double * linear,
                       const double * lower, const double * upper)
{
        if (!constraints || nrhs != sparse_matrix_nrows(constraints)
            || nvars != sparse_matrix_ncolumns(constraints) || (nrhs && !rhs)) {
                acd::set_error(ACDALM_EINVAL, "approx_make: shape mismatch or NULL rhs");
                return nullptr;
        }
        approx_t * a = new (std::nothrow) approx;
        if (!a)
                return nullptr;
        a->nrhs = nrhs;
        a->nvars = nvars;
        a->matrix = constraints;
        a->rhs = copy_or(rhs, nrhs, 0);
        a->weight = copy_or(weight, nrhs, 1);
        a->linear = copy_or(linear, nvars, 0);
        a->lower = copy_or(lower, nvars, -HUGE_VAL);
        a->upper = copy_or(upper, nvars, HUGE_VAL);
        a->permuted = sparse_matrix_copy(constraints, 1);
        if (!a->permuted) {
                delete a;
                return nullptr;
        }
        approx_update(a);
        return a;
}

int approx_free(approx_t * a)
{
        if (!a)
                return 0;
        if (a->dev_ready)
                a->dev.destroy();
        sparse_matrix_free(a->permuted);
        delete a;
        return 0;
}

sparse_matrix_t * approx_matrix(approx_t * a) { return a->matrix; }
size_t approx_nrhs(approx_t * a) { return a->nrhs; }
double * approx_rhs(approx_t * a) { return a->rhs.data(); }
double * approx_weight(approx_t * a) { return a->weight.data(); }
size_t approx_nvars(approx_t * a) { return a->nvars; }
double * approx_linear(approx_t * a) { return a->linear.data(); }
double * approx_lower(approx_t * a) { return a->lower.data(); }
double * approx_upper(approx_t * a) { return a->upper.data(); }

// approx.c:188-216: publish the live vectors to the shadow the solver reads
// (the step sizes are recomputed on the device at each solve from it).
int approx_update(approx_t * a)
{
        std::lock_guard<std::mutex> g(a->lock);
        a->s_rhs = a->rhs;
        a->s_weight = a->weight;
        a->s_linear = a->linear;
        a->s_lower = a->lower;
        a->s_upper = a->upper;
        return 0;
}

int approx_solve(double * x, size_t n, approx_t * a, size_t niter, double max_pg,
                 double max_value, double min_delta, FILE * log, size_t period,
                 double * OUT_diagnosis, double offset, thread_pool_t * pool)
{
        (void)pool;
        if (!a || n != a->nvars || (n && !x)) {
                acd::set_error(ACDALM_EINVAL, "approx_solve: n does not match the instance");
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(a->lock);
        int r = check_approx_inputs("approx_solve", a, x);
        if (r || (r = ensure_device(a)))
                return r;
        return acd::run_approx(a->dev, shadow_vectors(a), x, niter, max_pg, max_value,
                               min_delta, log, period, OUT_diagnosis, offset, a->stats);
}

int mpg_solve(double * x, size_t n, approx_t * a, size_t niter, double max_pg,
              double max_value, double min_delta, FILE * log, size_t period,
              double * OUT_diagnosis, double offset, thread_pool_t * pool)
{
        (void)pool;
        (void)min_delta;
        if (!a || n != a->nvars || (n && !x)) {
                acd::set_error(ACDALM_EINVAL, "mpg_solve: n does not match the instance");
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(a->lock);
        int r = check_approx_inputs("mpg_solve", a, x);
        if (r || (r = ensure_device(a)))
                return r;
        return acd::run_mpg(a->dev, shadow_vectors(a), x, niter, max_pg, max_value, log,
                            period, OUT_diagnosis, offset, a->stats);
}

// Same signature as the reference's serial randomized coordinate descent
// (approx/cd.c:332-385); runs APPROX on the GPU instead.
int cd_solve(double * x, size_t n, approx_t * a, size_t niter, double max_pg,
             double max_value, double min_delta, FILE * log, size_t period,
             double * OUT_diagnosis, double offset, thread_pool_t * pool)
{
        return approx_solve(x, n, a, niter, max_pg, max_value, min_delta, log, period,
                            OUT_diagnosis, offset, pool);
}

// ---- alm ----

alm_t * alm_make(sparse_matrix_t * constraints, size_t nrhs, const double * rhs,
                 size_t nvars, const double * linear, const double * lower,
                 const double * upper, const double * lambda_lower,
                 const double * lambda_upper)
{
        alm_t * m = new (std::nothrow) alm;
        if (!m)
                return nullptr;
        m->nrhs = nrhs;
        m->nvars = nvars;
        m->matrix = constraints;
        m->linear = copy_or(linear, nvars, 0);
        m->approx = approx_make(constraints, nrhs, rhs, nullptr, nvars, nullptr, lower,
                                upper);
        if (!m->approx) {
                delete m;
                return nullptr;
        }
        m->lambda_lower = copy_or(lambda_lower, nrhs, -HUGE_VAL);
        m->lambda_upper = copy_or(lambda_upper, nrhs, HUGE_VAL);
        return m;
}

int alm_free(alm_t * m)
{
        if (!m)
                return 0;
        approx_free(m->approx);
        delete m;
        return 0;
}

sparse_matrix_t * alm_matrix(alm_t * m) { return m->matrix; }
size_t alm_nrhs(alm_t * m) { return m->nrhs; }
double * alm_rhs(alm_t * m) { return approx_rhs(m->approx); }
size_t alm_nvars(alm_t * m) { return m->nvars; }
double * alm_linear(alm_t * m) { return m->linear.data(); }
double * alm_lower(alm_t * m) { return approx_lower(m->approx); }
double * alm_upper(alm_t * m) { return approx_upper(m->approx); }
double * alm_lambda_lower(alm_t * m) { return m->lambda_lower.data(); }
double * alm_lambda_upper(alm_t * m) { return m->lambda_upper.data(); }

int alm_solve(alm_t * m, size_t niter, double * x, size_t nvars, double * lambda,
              size_t nconstraints, FILE * log, double * OUT_diagnosis,
              thread_pool_t * pool)
{
        (void)pool;
        if (!m || nvars != m->nvars || nconstraints != m->nrhs || (nvars && !x)
            || (nconstraints && !lambda)) {
                acd::set_error(ACDALM_EINVAL, "alm_solve: sizes do not match the instance");
                return ACDALM_EINVAL;
        }
        approx_t * a = m->approx;
        std::lock_guard<std::mutex> g(a->lock);
        int r;
        if ((r = check_finite("alm_solve", "rhs", a->rhs.data(), m->nrhs, false))
            || (r = check_finite("alm_solve", "weight", a->weight.data(), m->nrhs, false))
            || (r = check_finite("alm_solve", "linear", m->linear.data(), m->nvars, false))
            || (r = check_finite("alm_solve", "lower", a->lower.data(), m->nvars, true))
            || (r = check_finite("alm_solve", "upper", a->upper.data(), m->nvars, true))
            || (r = check_finite("alm_solve", "lambda_lower", m->lambda_lower.data(), m->nrhs,
                                 true))
            || (r = check_finite("alm_solve", "lambda_upper", m->lambda_upper.data(), m->nrhs,
                                 true))
            || (r = check_finite("alm_solve", "x", x, m->nvars, false))
            || (r = check_finite("alm_solve", "lambda", lambda, m->nrhs, false)))
                return r;
        if ((r = ensure_device(a)))
                return r;
        // alm.c reads the live approx vectors each outer iteration
        acd::HostVectors hv;
        hv.b = a->rhs.data();
        hv.w = a->weight.data();
        hv.c0 = m->linear.data();
        hv.l = a->lower.data();
        hv.u = a->upper.data();
        hv.lam_lo = m->lambda_lower.data();
        hv.lam_hi = m->lambda_upper.data();
        r = acd::run_alm(a->dev, hv, niter, x, lambda, log, OUT_diagnosis, m->settings,
                         a->weight.data(), a->linear.data(), m->stats, &a->lay);
        if (r >= 0) {
                // the shadow holds what the last outer iteration published
                a->s_rhs = a->rhs;
                a->s_weight = a->weight;
                a->s_linear = a->linear;
                a->s_lower = a->lower;
                a->s_upper = a->upper;
        }
        return r;
}

alm_t * alm_read(FILE * stream)
{
        sparse_matrix_t * mat = sparse_matrix_read(stream, 0);
        if (!mat)
                return nullptr;
        size_t n = sparse_matrix_ncolumns(mat), mrows = sparse_matrix_nrows(mat);
        std::vector<double> rhs(mrows), lin(n), lo(n), hi(n), llo(mrows), lhi(mrows);
        auto rd = [&](std::vector<double> & v) {
                for (auto & e : v)
                        if (fscanf(stream, " %lf", &e) != 1)
                                return false;
                return true;
        };
        if (!rd(rhs) || !rd(lin) || !rd(lo) || !rd(hi) || !rd(llo) || !rd(lhi)) {
                acd::set_error(ACDALM_EINVAL, "alm_read: truncated vectors");
                sparse_matrix_free(mat);
                return nullptr;
        }
        return alm_make(mat, mrows, rhs.data(), n, lin.data(), lo.data(), hi.data(),
                        llo.data(), lhi.data());
}

}  // extern "C"

// ---- binary instances ----
//
// "ACDALMB1", then u64 nrows, ncols, nnz, then rows u32[nnz], columns
// u32[nnz], values f64[nnz], rhs f64[nrows], linear, lower, upper f64[ncols],
// dual lower, dual upper f64[nrows]; little-endian as the host writes it.
// The same content as alm_read's text (alm.c:330-364), without parsing.

namespace {

const char kBinaryMagic[8] = {'A', 'C', 'D', 'A', 'L', 'M', 'B', '1'};

template <class T>
bool put(FILE * f, const T * p, size_t n)
{
        return n == 0 || fwrite(p, sizeof(T), n, f) == n;
}

template <class T>
bool get(FILE * f, std::vector<T> & v, size_t n)
{
        v.resize(n);
        return n == 0 || fread(v.data(), sizeof(T), n, f) == n;
}

}  // namespace

extern "C" int acdalm_write_binary(alm_t * m, FILE * stream)
{
        if (!m || !stream) {
                acd::set_error(ACDALM_EINVAL, "acdalm_write_binary: null argument");
                return ACDALM_EINVAL;
        }
        sparse_matrix_t * a = alm_matrix(m);
        size_t nrows = alm_nrhs(m), ncols = alm_nvars(m), nnz = sparse_matrix_nnz(a);
        uint64_t hdr[3] = {nrows, ncols, nnz};
        bool ok = put(stream, kBinaryMagic, 8) && put(stream, hdr, 3)
                && put(stream, sparse_matrix_rows(a), nnz)
                && put(stream, sparse_matrix_columns(a), nnz)
                && put(stream, sparse_matrix_values(a), nnz)
                && put(stream, alm_rhs(m), nrows) && put(stream, alm_linear(m), ncols)
                && put(stream, alm_lower(m), ncols) && put(stream, alm_upper(m), ncols)
                && put(stream, alm_lambda_lower(m), nrows)
                && put(stream, alm_lambda_upper(m), nrows);
        if (!ok) {
                acd::set_error(ACDALM_EINVAL, "acdalm_write_binary: short write");
                return ACDALM_EINVAL;
        }
        return 0;
}

extern "C" alm_t * acdalm_read_binary(FILE * stream)
{
        char magic[8];
        uint64_t hdr[3];
        if (!stream || fread(magic, 1, 8, stream) != 8 || memcmp(magic, kBinaryMagic, 8) != 0
            || fread(hdr, sizeof(uint64_t), 3, stream) != 3) {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_binary: not an ACDALMB1 stream");
                return nullptr;
        }
        uint64_t nrows = hdr[0], ncols = hdr[1], nnz = hdr[2];
        if (nrows >= (1ull << 31) || ncols >= (1ull << 31) || nnz >= (1ull << 32)) {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_binary: sizes out of range");
                return nullptr;
        }
        std::vector<uint32_t> rows, cols;
        std::vector<double> vals, rhs, lin, lo, hi, llo, lhi;
        if (!get(stream, rows, nnz) || !get(stream, cols, nnz) || !get(stream, vals, nnz)
            || !get(stream, rhs, nrows) || !get(stream, lin, ncols) || !get(stream, lo, ncols)
            || !get(stream, hi, ncols) || !get(stream, llo, nrows) || !get(stream, lhi, nrows)) {
                acd::set_error(ACDALM_EINVAL, "acdalm_read_binary: truncated stream");
                return nullptr;
        }
        sparse_matrix_t * mat = sparse_matrix_make(ncols, nrows, nnz, rows.data(), cols.data(),
                                                   vals.data(), 0);
        if (!mat)
                return nullptr;
        alm_t * m = alm_make(mat, nrows, rhs.data(), ncols, lin.data(), lo.data(), hi.data(),
                             llo.data(), lhi.data());
        if (!m)
                sparse_matrix_free(mat);
        return m;
}

extern "C" {

// ---- extensions ----

int alm_set_precision(struct alm * m, int mode)
{
        if (mode != ACDALM_PRECISION_FP64 && mode != ACDALM_PRECISION_MIXED &&
            mode != ACDALM_PRECISION_AUTO) {
                acd::set_error(ACDALM_EINVAL, "alm_set_precision: mode %d", mode);
                return ACDALM_EINVAL;
        }
        m->settings.precision = mode;
        return 0;
}

int alm_set_kkt_tolerance(struct alm * m, double tol)
{
        if (!(tol >= 0)) {
                acd::set_error(ACDALM_EINVAL, "alm_set_kkt_tolerance: %g", tol);
                return ACDALM_EINVAL;
        }
        m->settings.kkt_tol = tol;
        return 0;
}

int alm_set_inner_budget(struct alm * m, uint64_t budget)
{
        m->settings.inner_budget = budget;
        return 0;
}

static void fill_stats(const acd::SolveStats & s, acdalm_stats_t * o)
{
        o->seconds = s.seconds;
        o->inner_iterations = s.inner;
        o->outer_iterations = s.outer;
        o->rel_kkt = s.rel_kkt;
        o->primal = s.primal;
        o->dual = s.dual;
        o->gap = s.gap;
        o->objective = s.objective;
        o->status = s.status;
        o->precision = s.precision;
        o->fp32_inner_iterations = s.inner_fp32;
}

int alm_last_stats(struct alm * m, acdalm_stats_t * out)
{
        fill_stats(m->stats, out);
        return 0;
}

int approx_last_stats(struct approx * a, acdalm_stats_t * out)
{
        fill_stats(a->stats, out);
        return 0;
}

void * alm_stream(struct alm * m)
{
        return approx_stream(m->approx);
}

void * approx_stream(struct approx * a)
{
        if (ensure_device(a))
                return nullptr;
        return (void *)a->dev.stream;
}

struct approx * acdalm_alm_approx(struct alm * m)
{
        return m->approx;
}

struct sparse_matrix * acdalm_approx_permuted_matrix(struct approx * a)
{
        return a->permuted;
}

// ---- batches ----

acdalm_batch_t * acdalm_batch_make(struct alm * const * instances, size_t count)
{
        if (count && !instances) {
                acd::set_error(ACDALM_EINVAL, "acdalm_batch_make: NULL instances");
                return nullptr;
        }
        for (size_t i = 0; i < count; i++)
                if (!instances[i]) {
                        acd::set_error(ACDALM_EINVAL, "acdalm_batch_make: instance %zu is NULL", i);
                        return nullptr;
                }
        acdalm_batch_t * b = new (std::nothrow) acdalm_batch;
        if (!b)
                return nullptr;
        b->alms.assign(instances, instances + count);
        // one CTA per LP: device layouts not built yet are built for it
        // (full lanes, no step cap); instances already solved keep theirs
        for (size_t i = 0; i < count; i++) {
                approx_t * a = instances[i]->approx;
                std::lock_guard<std::mutex> g(a->lock);
                if (!a->lay_ready)
                        a->lay_max_steps = 0;
        }
        return b;
}

int acdalm_batch_free(acdalm_batch_t * b)
{
        delete b;
        return 0;
}

int acdalm_batch_solve(acdalm_batch_t * b, size_t niter, double * const * x,
                       double * const * lambda, int * ret, double * diag)
{
        if (!b || (b->alms.size() && (!x || !lambda))) {
                acd::set_error(ACDALM_EINVAL, "acdalm_batch_solve: NULL arguments");
                return ACDALM_EINVAL;
        }
        size_t n = b->alms.size();
        std::vector<acd::BatchEntry> entries(n);
        std::vector<std::unique_lock<std::mutex>> locks;
        for (size_t i = 0; i < n; i++) {
                alm_t * m = b->alms[i];
                approx_t * a = m->approx;
                locks.emplace_back(a->lock);
                int r = ensure_device(a);
                if (r)
                        return r;
                acd::BatchEntry & e = entries[i];
                e.dev = &a->dev;
                e.lay = &a->lay;
                e.hv.b = a->rhs.data();
                e.hv.w = a->weight.data();
                e.hv.c0 = m->linear.data();
                e.hv.l = a->lower.data();
                e.hv.u = a->upper.data();
                e.hv.lam_lo = m->lambda_lower.data();
                e.hv.lam_hi = m->lambda_upper.data();
                e.settings = m->settings;
                e.x = x[i];
                e.lam = lambda[i];
                e.diag3 = diag ? diag + 3 * i : nullptr;
                e.w_out = a->weight.data();
                e.c_out = a->linear.data();
                e.stats = &m->stats;
        }
        int r = acd::run_alm_batch(entries, niter, &b->seconds);
        for (size_t i = 0; i < n; i++) {
                if (ret)
                        ret[i] = entries[i].ret;
                approx_t * a = b->alms[i]->approx;
                if (entries[i].ret >= 0) {
                        a->s_rhs = a->rhs;
                        a->s_weight = a->weight;
                        a->s_linear = a->linear;
                        a->s_lower = a->lower;
                        a->s_upper = a->upper;
                }
        }
        return r;
}

double acdalm_batch_seconds(acdalm_batch_t * b)
{
        return b ? b->seconds : 0;
}

int alm_set_trace(struct alm * m, uint64_t first, uint64_t count)
{
        if (!m || first > 0xffffffffull || count > (1u << 20)) {
                acd::set_error(ACDALM_EINVAL, "alm_set_trace: reductions %llu + %llu",
                               (unsigned long long)first, (unsigned long long)count);
                return ACDALM_EINVAL;
        }
        m->settings.trace_first = (unsigned)first;
        m->settings.trace_count = (unsigned)count;
        return 0;
}

int alm_trace_copy(struct alm * m, uint64_t * out, size_t cap, size_t * ctas, size_t * count)
{
        if (!m) {
                acd::set_error(ACDALM_EINVAL, "alm_trace_copy: NULL instance");
                return ACDALM_EINVAL;
        }
        approx_t * a = m->approx;
        std::lock_guard<std::mutex> g(a->lock);
        if (!a->dev_ready) {
                if (ctas)
                        *ctas = 0;
                if (count)
                        *count = 0;
                return 0;
        }
        return acd::copy_trace(a->dev, reinterpret_cast<unsigned long long *>(out), cap, ctas,
                               count);
}

// Step sizes as the solver computes them, in original order: beta (m), v,
// inv_v (n).  For the parity tests of approx.c:135-186.
int acdalm_approx_step_sizes(struct approx * a, double * beta, double * v, double * inv_v)
{
        std::lock_guard<std::mutex> g(a->lock);
        int r = ensure_device(a);
        if (r)
                return r;
        return acd::dev_step_sizes(a->dev, shadow_vectors(a), beta, v, inv_v);
}

}  // extern "C"
