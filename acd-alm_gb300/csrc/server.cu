// acdalm_server: continuous batching of LP solves on one GPU.
//
// Requests (an LP each) are submitted at any time.  A pool of builder
// threads turns each into its host layouts (the permuted copy and the
// device layout), one-CTA requests before larger ones (a larger one that
// has waited kBackfillSeconds goes next).  A dispatcher thread admits built
// requests: each admitted LP gets its device instance, its data uploaded,
// and one solve launched on its own stream -- one CTA for a small LP, a
// thread-block cluster of up to 16 CTAs for a large one -- so LPs that
// arrive while others are on the GPU run beside them.  Finished solves are
// retired (results read back, device memory freed), which frees SMs and
// budget for the next requests.
//
// Admission packs the GPU's SMs (admission.h): a request is admitted only
// while the running teams leave enough SMs free for its team, its device
// footprint fits the memory budget and fewer than max_inflight solves run,
// so no admitted solve waits in the hardware queue holding a slot; one-CTA
// requests go first, then clusters with the most nonzeros, and smaller
// requests fill SMs a larger one cannot use yet until it has waited
// kBackfillSeconds.  Clusters run on high-priority streams: a cluster's
// CTAs must all find room in one GPC at once.  Every solve is the same
// computation whether it runs alone or in the mix (a fixed team,
// deterministic reductions).
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/acdalm_ext.h"
#include "../../include/alm.h"
#include "admission.h"
#include "common.h"
#include "instance.h"
#include "layout.h"
#include "objects.h"

namespace acd {
HostMatrix & host_of(sparse_matrix_t * m);
}

namespace {

using Clock = std::chrono::steady_clock;

// How long a built request may be passed by smaller ones that fit the free
// SMs before it blocks them (see the admission rule above).
constexpr double kBackfillSeconds = 10.0;

enum State { PENDING, BUILT, RUNNING, DONE, FAILED };

struct Request {
        long long id = 0;
        size_t m = 0, n = 0, nnz = 0;
        std::vector<uint32_t> rows, cols;
        std::vector<double> vals, rhs, linear, lower, upper, llo, lhi;
        sparse_matrix_t * matrix = nullptr;
        alm_t * alm = nullptr;
        size_t footprint = 0;
        int team = 1;  // CTAs (a thread-block cluster) solving this LP
        acd::AlmLaunch launch;
        std::vector<double> x, lam;
        double diag[3] = {0, 0, 0};
        acd::SolveStats stats;
        int ret = 0;
        State state = PENDING;
        Clock::time_point t_submit, t_built, t_admit, t_done;
};

}  // namespace

struct acdalm_server {
        size_t budget = 0;         // device bytes for admitted instances
        int max_team = 16;         // largest cluster the device launches
        int sms = 0;               // SMs of the device
        int sms_busy = 0;          // SMs the running solves' teams hold
        size_t in_use = 0;
        int max_inflight = 0;
        int precision = 0;
        int high_priority = 0;     // stream priority of cluster solves
        double kkt_tol = 1e-6;
        size_t niter = 1000;
        unsigned long long inner_budget = 0;

        std::mutex mu;
        std::condition_variable cv_build, cv_done;
        std::map<long long, std::unique_ptr<Request>> reqs;
        // submitted, not built: LPs a single CTA solves, and the rest
        std::deque<Request *> to_build_small, to_build_large;
        std::deque<Request *> built;     // built, not admitted (arrival order)
        std::vector<Request *> running;
        std::deque<long long> finished;  // retired, not yet polled
        long long next_id = 0;
        bool stop = false;
        std::vector<std::thread> builders;
        std::thread dispatcher;
        std::atomic<long long> completed{0};
        std::string error;
};

namespace {

// A built request as the admission rule sees it at time `now`.
acd::Candidate candidate(const Request * r, Clock::time_point now)
{
        acd::Candidate c;
        c.id = r->id;
        c.nnz = r->nnz;
        c.team = r->team;
        c.footprint = r->footprint;
        c.waited = std::chrono::duration<double>(now - r->t_built).count();
        return c;
}

// Cluster size (CTAs per LP) for an LP with nnz nonzeros.
int team_size(long long nnz)
{
        if (nnz <= 150000)
                return 1;
        if (nnz <= 600000)
                return 4;
        if (nnz <= 1500000)
                return 8;
        return 16;
}

void build_one(acdalm_server_t * s, Request * r)
{
        r->matrix = sparse_matrix_make(r->n, r->m, r->vals.size(), r->rows.data(),
                                       r->cols.data(), r->vals.data(), 0);
        if (r->matrix)
                r->alm = alm_make(r->matrix, r->m, r->rhs.data(), r->n, r->linear.data(),
                                  r->lower.data(), r->upper.data(), r->llo.data(),
                                  r->lhi.data());
        if (r->alm) {
                approx_t * a = r->alm->approx;
                acd::build_device_layout(acd::host_of(a->permuted), a->lay, 0);
                a->lay_ready = true;
                r->team = std::min(team_size((long long)r->vals.size()), s->max_team);
                // the COO copies are not needed any more
                std::vector<uint32_t>().swap(r->rows);
                std::vector<uint32_t>().swap(r->cols);
                std::vector<double>().swap(r->vals);
        }
        std::lock_guard<std::mutex> g(s->mu);
        if (!r->alm) {
                r->state = FAILED;
                r->ret = ACDALM_EINVAL;
                r->t_done = Clock::now();
                s->finished.push_back(r->id);
                s->cv_done.notify_all();
                return;
        }
        approx_t * a = r->alm->approx;
        r->alm->settings.kkt_tol = s->kkt_tol;
        r->alm->settings.precision = s->precision;
        r->alm->settings.inner_budget = s->inner_budget;
        r->footprint = acd::DevInstance::footprint(a->lay,
                                                   acd::mixed_for(s->precision, a->lay.nnz));
        r->state = BUILT;
        r->t_built = Clock::now();
        // keep the built queue in admission order
        auto it = s->built.begin();
        while (it != s->built.end() && acd::admits_before(candidate(*it, r->t_built),
                                                          candidate(r, r->t_built)))
                ++it;
        s->built.insert(it, r);
}

void builder_main(acdalm_server_t * s)
{
        for (;;) {
                Request * r;
                {
                        std::unique_lock<std::mutex> g(s->mu);
                        s->cv_build.wait(g, [&] {
                                return s->stop || !s->to_build_small.empty() ||
                                       !s->to_build_large.empty();
                        });
                        if (s->stop)
                                return;
                        // one-CTA requests first (they are admitted first,
                        // and their builds are short), unless a larger one
                        // has waited longer than the backfill limit
                        bool large = !s->to_build_large.empty() &&
                                     (s->to_build_small.empty() ||
                                      std::chrono::duration<double>(
                                              Clock::now() - s->to_build_large.front()->t_submit)
                                                      .count() > kBackfillSeconds);
                        std::deque<Request *> & q = large ? s->to_build_large : s->to_build_small;
                        r = q.front();
                        q.pop_front();
                }
                build_one(s, r);
        }
}

// Admission and retirement; the only thread that touches the GPU.
void dispatcher_main(acdalm_server_t * s)
{
        acd::device_ready();
        for (;;) {
                bool idle = true;
                // retire finished solves
                std::vector<Request *> done_now;
                {
                        std::lock_guard<std::mutex> g(s->mu);
                        for (size_t i = 0; i < s->running.size();) {
                                Request * r = s->running[i];
                                if (cudaEventQuery(r->launch.done) == cudaSuccess) {
                                        done_now.push_back(r);
                                        s->running[i] = s->running.back();
                                        s->running.pop_back();
                                } else {
                                        i++;
                                }
                        }
                }
                for (Request * r : done_now) {
                        idle = false;
                        approx_t * a = r->alm->approx;
                        r->x.assign(r->n, 0.0);
                        r->lam.assign(r->m, 0.0);
                        r->ret = acd::alm_collect(a->dev, r->launch, r->x.data(), r->lam.data(),
                                                  r->diag, r->stats);
                        alm_free(r->alm);
                        sparse_matrix_free(r->matrix);
                        r->alm = nullptr;
                        r->matrix = nullptr;
                        std::lock_guard<std::mutex> g(s->mu);
                        r->t_done = Clock::now();
                        r->state = r->ret < 0 ? FAILED : DONE;
                        s->in_use -= r->footprint;
                        s->sms_busy -= r->team;
                        s->finished.push_back(r->id);
                        s->completed++;
                        s->cv_done.notify_all();
                }
                // admit built requests while SMs, memory and slots allow
                for (;;) {
                        Request * r = nullptr;
                        {
                                std::lock_guard<std::mutex> g(s->mu);
                                if (s->built.empty() || (int)s->running.size() >= s->max_inflight)
                                        break;
                                bool nothing_running = s->running.empty();
                                auto now = Clock::now();
                                acd::Capacity cap;
                                cap.sms = s->sms;
                                cap.sms_busy = s->sms_busy;
                                cap.budget = s->budget;
                                cap.in_use = s->in_use;
                                cap.nothing_running = nothing_running;
                                cap.backfill_seconds = kBackfillSeconds;
                                long at = acd::pick_admission(
                                        s->built.size(),
                                        [&](size_t i) { return candidate(s->built[i], now); }, cap);
                                if (at < 0)
                                        break;
                                auto pick = s->built.begin() + at;
                                Request * head = *pick;
                                if (head->footprint > s->budget && nothing_running) {
                                        // can never fit: fail it rather than stall
                                        s->built.erase(pick);
                                        head->state = FAILED;
                                        head->ret = ACDALM_ENOMEM;
                                        head->t_done = Clock::now();
                                        s->finished.push_back(head->id);
                                        s->cv_done.notify_all();
                                        continue;
                                }
                                s->built.erase(pick);
                                s->in_use += head->footprint;
                                s->sms_busy += head->team;
                                r = head;
                        }
                        idle = false;
                        approx_t * a = r->alm->approx;
                        alm_t * m = r->alm;
                        a->dev.priority = r->team > 1 ? s->high_priority : 0;
                        int e = a->dev.create(a->lay);
                        if (!e)
                                a->dev_ready = true;
                        r->t_admit = Clock::now();
                        r->x.assign(r->n, 0.0);
                        r->lam.assign(r->m, 0.0);
                        if (!e) {
                                acd::HostVectors hv;
                                hv.b = a->rhs.data();
                                hv.w = a->weight.data();
                                hv.c0 = m->linear.data();
                                hv.l = a->lower.data();
                                hv.u = a->upper.data();
                                hv.lam_lo = m->lambda_lower.data();
                                hv.lam_hi = m->lambda_upper.data();
                                e = acd::alm_launch_async(a->dev, hv, s->niter, r->x.data(),
                                                          r->lam.data(), m->settings, &a->lay,
                                                          r->launch, r->team);
                        }
                        std::lock_guard<std::mutex> g(s->mu);
                        if (e) {
                                r->state = FAILED;
                                r->ret = e;
                                r->t_done = Clock::now();
                                s->in_use -= r->footprint;
                                s->sms_busy -= r->team;
                                s->finished.push_back(r->id);
                                s->cv_done.notify_all();
                        } else {
                                r->state = RUNNING;
                                s->running.push_back(r);
                        }
                }
                {
                        std::lock_guard<std::mutex> g(s->mu);
                        if (s->stop && s->running.empty())
                                return;
                }
                if (idle)
                        std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
}

}  // namespace

extern "C" {

acdalm_server_t * acdalm_server_create(size_t device_budget, int max_inflight, int precision,
                                       double kkt_tol, int builder_threads)
{
        if (precision < 0 || precision > 2) {
                acd::set_error(ACDALM_EINVAL, "acdalm_server_create: precision mode %d",
                               precision);
                return nullptr;
        }
        if (!acd::device_ready())
                return nullptr;
        acdalm_server_t * s = new (std::nothrow) acdalm_server;
        if (!s)
                return nullptr;
        if (device_budget == 0) {
                size_t free_b = 0, total_b = 0;
                cudaMemGetInfo(&free_b, &total_b);
                device_budget = free_b / 10 * 8;
        }
        s->budget = device_budget;
        s->max_team = acd::max_cluster_team();
        {
                int dev = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
                s->sms = std::max(s->sms, s->max_team);
        }
        s->max_inflight = max_inflight > 0 ? max_inflight : 128;
        s->precision = precision;
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess)
                s->high_priority = greatest;
        s->kkt_tol = kkt_tol;
        int nb = builder_threads > 0 ? builder_threads
                                     : std::max(1u, std::thread::hardware_concurrency() / 2);
        for (int i = 0; i < nb; i++)
                s->builders.emplace_back(builder_main, s);
        s->dispatcher = std::thread(dispatcher_main, s);
        return s;
}

int acdalm_server_set_inner_budget(acdalm_server_t * s, uint64_t budget)
{
        if (!s) {
                acd::set_error(ACDALM_EINVAL, "acdalm_server_set_inner_budget: NULL server");
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(s->mu);
        s->inner_budget = budget;
        return 0;
}

long long acdalm_server_submit(acdalm_server_t * s, size_t nrows, size_t ncols, size_t nnz,
                               const uint32_t * rows, const uint32_t * cols,
                               const double * vals, const double * rhs, const double * linear,
                               const double * lower, const double * upper,
                               const double * lambda_lower, const double * lambda_upper)
{
        if (!s || (nnz && (!rows || !cols || !vals)) || (nrows && !rhs)) {
                acd::set_error(ACDALM_EINVAL, "acdalm_server_submit: bad arguments");
                return ACDALM_EINVAL;
        }
        auto r = std::make_unique<Request>();
        r->m = nrows;
        r->n = ncols;
        r->nnz = nnz;
        r->rows.assign(rows, rows + nnz);
        r->cols.assign(cols, cols + nnz);
        r->vals.assign(vals, vals + nnz);
        r->rhs.assign(rhs, rhs + nrows);
        auto vec = [](const double * p, size_t n, double dflt) {
                std::vector<double> v(n);
                for (size_t i = 0; i < n; i++)
                        v[i] = p ? p[i] : dflt;
                return v;
        };
        r->linear = vec(linear, ncols, 0);
        r->lower = vec(lower, ncols, -HUGE_VAL);
        r->upper = vec(upper, ncols, HUGE_VAL);
        r->llo = vec(lambda_lower, nrows, -HUGE_VAL);
        r->lhi = vec(lambda_upper, nrows, HUGE_VAL);
        r->t_submit = Clock::now();
        std::lock_guard<std::mutex> g(s->mu);
        long long id = s->next_id++;
        r->id = id;
        (team_size((long long)nnz) == 1 ? s->to_build_small : s->to_build_large)
                .push_back(r.get());
        s->reqs[id] = std::move(r);
        s->cv_build.notify_one();
        return id;
}

int acdalm_server_poll(acdalm_server_t * s, long long * ids, int cap, double timeout)
{
        std::unique_lock<std::mutex> g(s->mu);
        if (s->finished.empty() && timeout > 0)
                s->cv_done.wait_for(g, std::chrono::duration<double>(timeout),
                                    [&] { return !s->finished.empty(); });
        int n = 0;
        while (n < cap && !s->finished.empty()) {
                ids[n++] = s->finished.front();
                s->finished.pop_front();
        }
        return n;
}

int acdalm_server_result(acdalm_server_t * s, long long id, double * x, double * lambda,
                         acdalm_stats_t * st, double * latency)
{
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) {
                acd::set_error(ACDALM_EINVAL, "acdalm_server_result: unknown id %lld", id);
                return ACDALM_EINVAL;
        }
        Request * r = it->second.get();
        if (r->state != DONE && r->state != FAILED) {
                acd::set_error(ACDALM_EINVAL, "acdalm_server_result: request %lld not finished", id);
                return ACDALM_EINVAL;
        }
        if (x && !r->x.empty())
                std::copy(r->x.begin(), r->x.end(), x);
        if (lambda && !r->lam.empty())
                std::copy(r->lam.begin(), r->lam.end(), lambda);
        if (st) {
                memset(st, 0, sizeof(*st));
                st->seconds = std::chrono::duration<double>(r->t_done - r->t_admit).count();
                st->inner_iterations = r->stats.inner;
                st->outer_iterations = r->stats.outer;
                st->rel_kkt = r->stats.rel_kkt;
                st->primal = r->stats.primal;
                st->dual = r->stats.dual;
                st->gap = r->stats.gap;
                st->objective = r->stats.objective;
                st->status = r->ret < 0 ? r->ret : r->stats.status;
                st->precision = r->stats.precision;
                st->fp32_inner_iterations = r->stats.inner_fp32;
        }
        if (latency)
                *latency = std::chrono::duration<double>(r->t_done - r->t_submit).count();
        int ret = r->ret;
        s->reqs.erase(it);
        return ret;
}

int acdalm_server_destroy(acdalm_server_t * s)
{
        if (!s)
                return 0;
        {
                std::lock_guard<std::mutex> g(s->mu);
                s->stop = true;
        }
        s->cv_build.notify_all();
        for (auto & t : s->builders)
                t.join();
        s->dispatcher.join();
        for (auto & kv : s->reqs) {
                Request * r = kv.second.get();
                if (r->alm)
                        alm_free(r->alm);
                if (r->matrix)
                        sparse_matrix_free(r->matrix);
        }
        delete s;
        return 0;
}

}  // extern "C"
