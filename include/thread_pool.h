/* Host thread pool: the parallel-for / map-reduce runtime whose handle every
 * hot signature of the solver takes.
 *
 * Same entry points, argument meaning and return conventions as the
 * reference's thread_pool/thread_pool.h:8-89.  In libacdalm the solve loop
 * runs on the GPU, so the pool only parallelises host-side work (layout
 * builders); passing NULL everywhere is always valid.
 */
#ifndef ACDALM_THREAD_POOL_H
#define ACDALM_THREAD_POOL_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* NULL means serial execution. */
typedef struct thread_pool thread_pool_t;

/* A pool of nworker workers, the caller counting as worker 0 (so
 * nworker - 1 threads are started); 0 is treated as 1.
 * Replaces thread_pool_init, thread_pool/thread_pool.h:13. */
thread_pool_t * thread_pool_init(unsigned nworker);
/* Stops the workers and frees the pool; NULL is ignored (:15). */
void thread_pool_free(thread_pool_t *);
/* Number of workers including the caller (:19). */
size_t thread_pool_count(thread_pool_t *);
/* char_per_worker zeroed bytes for each worker, each on its own cache
 * line(s); the returned array is reused by later calls and freed with the
 * pool.  0 releases the storage (:31-32). */
void * const * thread_pool_worker_storage(thread_pool_t *,
                                          size_t char_per_worker);
/* The same storage as one flat buffer; *OUT_aligned_size (if non-NULL)
 * receives the padded per-worker size (:36-38). */
void * thread_pool_worker_storage_flat(thread_pool_t *,
                                       size_t char_per_worker,
                                       size_t * OUT_aligned_size);
/* Park the workers on a condition variable / wake them (:46-47). */
void thread_pool_sleep(thread_pool_t *);
void thread_pool_wakeup(thread_pool_t *);

/* Calls function(begin, end, info, worker_id) over disjoint subranges
 * covering [from, end); each subrange is a multiple of granularity (but the
 * last), scaled up to about 10 subranges per worker (:63-67). */
typedef void (*thread_pool_function)(size_t begin, size_t end, void * info,
                                     unsigned worker_id);
void thread_pool_for(thread_pool_t *,
                     size_t from, size_t end, size_t granularity,
                     thread_pool_function function, void * info);

/* As thread_pool_for, reducing the returned doubles with SUM, MAX or MIN
 * starting from initial_value (:80-89). */
typedef double (*thread_pool_map)(size_t begin, size_t end, void * info,
                                  unsigned worker_id);
enum thread_pool_reducer {THREAD_POOL_REDUCE_SUM,
                          THREAD_POOL_REDUCE_MAX,
                          THREAD_POOL_REDUCE_MIN};
double thread_pool_map_reduce(thread_pool_t *,
                              size_t from, size_t end, size_t granularity,
                              thread_pool_map function, void * info,
                              enum thread_pool_reducer reducer,
                              double initial_value);
#ifdef __cplusplus
}
#endif
#endif
