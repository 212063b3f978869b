// Host thread pool with the reference's interface (thread_pool/thread_pool.h).
// Workers block on a condition variable between jobs (no spinning); a job
// hands out subranges from an atomic cursor, as thread_pool.c:191-243 does.
#include "../../include/thread_pool.h"

#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

struct thread_pool {
        unsigned nworker = 1;
        std::vector<std::thread> threads;
        std::mutex mu;
        std::condition_variable cv, done_cv;
        bool stop = false;
        unsigned long long epoch = 0;
        // current job
        thread_pool_function fn = nullptr;
        void * info = nullptr;
        size_t from = 0, end = 0, grain = 1;
        std::atomic<size_t> cursor{0};
        unsigned active = 0;
        // worker storage
        void * storage = nullptr;
        size_t storage_stride = 0;
        std::vector<void *> storage_ptrs;
        std::atomic<bool> busy{false};
};

namespace {

void run_chunks(thread_pool_t * p, unsigned id)
{
        for (;;) {
                size_t b = p->cursor.fetch_add(p->grain);
                if (b >= p->end)
                        break;
                size_t e = (p->end - b < p->grain) ? p->end : b + p->grain;
                p->fn(b, e, p->info, id);
        }
}

void worker_main(thread_pool_t * p, unsigned id)
{
        unsigned long long seen = 0;
        for (;;) {
                std::unique_lock<std::mutex> g(p->mu);
                p->cv.wait(g, [&] { return p->stop || p->epoch != seen; });
                if (p->stop)
                        return;
                seen = p->epoch;
                g.unlock();
                run_chunks(p, id);
                g.lock();
                if (--p->active == 0)
                        p->done_cv.notify_all();
        }
}

// thread_pool.c:296-302: at least `minimum`, about 10 chunks per worker.
size_t ideal_granularity(size_t n, size_t minimum, unsigned workers)
{
        if (minimum == 0)
                minimum = 1;
        n = (n + minimum - 1) / minimum;
        size_t nchunks = (size_t)workers * 10;
        if (n < nchunks)
                return minimum;
        return minimum * ((n + nchunks - 1) / nchunks);
}

}  // namespace

extern "C" {

thread_pool_t * thread_pool_init(unsigned nworker)
{
        thread_pool_t * p = new thread_pool;
        p->nworker = nworker ? nworker : 1;
        for (unsigned i = 1; i < p->nworker; i++)
                p->threads.emplace_back(worker_main, p, i);
        return p;
}

void thread_pool_free(thread_pool_t * p)
{
        if (!p)
                return;
        {
                std::lock_guard<std::mutex> g(p->mu);
                p->stop = true;
        }
        p->cv.notify_all();
        for (auto & t : p->threads)
                t.join();
        free(p->storage);
        delete p;
}

size_t thread_pool_count(thread_pool_t * p)
{
        return p ? p->nworker : 1;
}

void * thread_pool_worker_storage_flat(thread_pool_t * p, size_t per_worker,
                                       size_t * out_aligned)
{
        size_t n = thread_pool_count(p);
        size_t stride = (per_worker + 63) & ~size_t(63);
        if (out_aligned)
                *out_aligned = stride;
        if (!p)
                return nullptr;
        free(p->storage);
        p->storage = nullptr;
        p->storage_stride = stride;
        if (per_worker == 0)
                return nullptr;
        p->storage = aligned_alloc(64, stride * n);
        memset(p->storage, 0, stride * n);
        return p->storage;
}

void * const * thread_pool_worker_storage(thread_pool_t * p, size_t per_worker)
{
        if (!p)
                return nullptr;
        char * base = (char *)thread_pool_worker_storage_flat(p, per_worker, nullptr);
        p->storage_ptrs.assign(p->nworker, nullptr);
        if (base)
                for (unsigned i = 0; i < p->nworker; i++)
                        p->storage_ptrs[i] = base + i * p->storage_stride;
        return p->storage_ptrs.data();
}

void thread_pool_sleep(thread_pool_t * p)
{
        (void)p;  // workers always sleep between jobs
}

void thread_pool_wakeup(thread_pool_t * p)
{
        (void)p;
}

void thread_pool_for(thread_pool_t * p, size_t from, size_t end, size_t granularity,
                     thread_pool_function function, void * info)
{
        if (!p || p->nworker <= 1 || end - from <= granularity) {
                function(from, end, info, 0);
                return;
        }
        {
                std::lock_guard<std::mutex> g(p->mu);
                p->fn = function;
                p->info = info;
                p->from = from;
                p->end = end;
                p->grain = ideal_granularity(end - from, granularity, p->nworker);
                p->cursor.store(from);
                p->active = p->nworker - 1;
                p->epoch++;
        }
        p->cv.notify_all();
        run_chunks(p, 0);
        std::unique_lock<std::mutex> g(p->mu);
        p->done_cv.wait(g, [&] { return p->active == 0; });
}

struct map_reduce_info {
        thread_pool_map fn;
        void * info;
        enum thread_pool_reducer red;
        double * acc;
        size_t stride;
};

static void map_reduce_worker(size_t b, size_t e, void * thunk, unsigned id)
{
        map_reduce_info * m = (map_reduce_info *)thunk;
        double v = m->fn(b, e, m->info, id);
        double * a = (double *)((char *)m->acc + id * m->stride);
        switch (m->red) {
        case THREAD_POOL_REDUCE_SUM: *a += v; break;
        case THREAD_POOL_REDUCE_MAX: *a = fmax(*a, v); break;
        default: *a = fmin(*a, v); break;
        }
}

double thread_pool_map_reduce(thread_pool_t * p, size_t from, size_t end,
                              size_t granularity, thread_pool_map function,
                              void * info, enum thread_pool_reducer reducer,
                              double initial_value)
{
        if (!p)
                return function(from, end, info, 0);
        size_t n = p->nworker, stride = 64;
        std::vector<double> accs(n * (stride / sizeof(double)), initial_value);
        map_reduce_info m = {function, info, reducer, accs.data(), stride};
        thread_pool_for(p, from, end, granularity, map_reduce_worker, &m);
        double acc = initial_value;
        for (size_t i = 0; i < n; i++) {
                double v = accs[i * (stride / sizeof(double))];
                switch (reducer) {
                case THREAD_POOL_REDUCE_SUM: acc += v; break;
                case THREAD_POOL_REDUCE_MAX: acc = fmax(acc, v); break;
                default: acc = fmin(acc, v); break;
                }
        }
        return acc;
}

}  // extern "C"
