// The LP server's admission rule (server.cu), kept free of CUDA so that the
// host tests can compile and check it on its own.
//
// Every admitted solve holds `team` SMs (one CTA per SM) until it ends.  A
// built request is admitted while the running teams leave enough SMs free
// for its team and its device footprint fits the memory budget.  Requests
// are taken in this order: one-CTA requests first, in arrival order (they
// are most requests and little of the work, so running them first cuts the
// typical latency at almost no cost to the end of a stream), then cluster
// requests with the most nonzeros first (a large LP started late sets the
// end of the whole stream), ties by arrival.  The first request in that
// order that fits goes next, so smaller ones fill SMs a larger one cannot
// use yet -- until a request has waited longer than the backfill limit,
// after which nothing behind it is admitted before it.
#pragma once
#include <cstddef>

namespace acd {

// What the rule needs to know of a built request.
struct Candidate {
        long long id = 0;     // arrival order
        size_t nnz = 0;
        int team = 1;         // SMs its solve holds
        size_t footprint = 0; // device bytes
        double waited = 0;    // seconds since it was built
};

// The GPU's state at the decision.
struct Capacity {
        int sms = 0, sms_busy = 0;
        size_t budget = 0, in_use = 0;
        bool nothing_running = false;
        double backfill_seconds = 10.0;
};

// True when p goes before q in the admission order.
inline bool admits_before(const Candidate & p, const Candidate & q)
{
        bool ps = p.team == 1, qs = q.team == 1;
        if (ps != qs)
                return ps;
        if (!ps && p.nnz != q.nnz)
                return p.nnz > q.nnz;
        return p.id < q.id;
}

// Index of the request to admit next among count requests already in
// admission order (get(i) gives the i-th as a Candidate), or -1 for none.
// With nothing running the first request is taken whatever its size (the
// caller fails one that can never fit rather than stall).
template <class Get>
inline long pick_admission(size_t count, Get && get, const Capacity & c)
{
        for (size_t i = 0; i < count; i++) {
                const Candidate q = get(i);
                bool fits = c.nothing_running ||
                            (c.sms_busy + q.team <= c.sms && c.in_use + q.footprint <= c.budget);
                if (fits)
                        return (long)i;
                if (q.waited > c.backfill_seconds)
                        return -1;
        }
        return -1;
}

}  // namespace acd
