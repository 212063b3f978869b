// Autotuner of the whole-GPU solve's device layout.
//
// A solve on the whole GPU waits, at every pass, for its slowest warp, and a
// warp's time is its chain of dependent steps; how many lanes share a row
// (which sets the steps per slice) trades that chain against lane
// utilisation, and where the balance lies depends on the LP's row and
// column lengths.  acdalm_autotune builds the instance's SELL layout with
// each candidate step cap, times a fixed number of APPROX iterations on the
// device with each, and keeps the fastest.  The choice is remembered for
// the instance's size class (row, column and nonzero counts in half-octave
// buckets), so later instances of that class skip the timing.
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/acdalm_ext.h"
#include "common.h"
#include "instance.h"
#include "layout.h"
#include "objects.h"

namespace acd {
HostMatrix & host_of(sparse_matrix_t * m);
}

namespace {

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, int> g_tuned;  // size class -> step cap

const int kCandidates[] = {0, 4, 8, 12, 16};

int size_class(double v)
{
        return (int)std::lround(2.0 * std::log2(v < 1 ? 1.0 : v));
}

}  // namespace

extern "C" int acdalm_autotune(struct alm * m, size_t iterations, int * chosen)
{
        if (!m || iterations == 0) {
                acd::set_error(ACDALM_EINVAL, "acdalm_autotune: NULL instance or no iterations");
                return ACDALM_EINVAL;
        }
        approx_t * a = m->approx;
        std::lock_guard<std::mutex> g(a->lock);
        if (!acd::device_ready())
                return ACDALM_ENODEV;
        acd::HostMatrix & host = acd::host_of(a->permuted);
        auto key = std::make_tuple(size_class((double)m->nrhs), size_class((double)m->nvars),
                                   size_class((double)host.nnz));
        int best = -1;
        {
                std::lock_guard<std::mutex> tg(g_tune_mu);
                auto it = g_tuned.find(key);
                if (it != g_tuned.end())
                        best = it->second;
        }
        if (best < 0) {
                // the instance's own problem: the ALM objective, current weights
                acd::HostVectors hv;
                hv.b = a->rhs.data();
                hv.w = a->weight.data();
                hv.c0 = m->linear.data();
                hv.l = a->lower.data();
                hv.u = a->upper.data();
                double best_s = HUGE_VAL;
                for (int cap : kCandidates) {
                        acd::DeviceLayout lay;
                        acd::build_device_layout(host, lay, cap);
                        acd::DevInstance d;
                        int r = d.create(lay);
                        double sec = HUGE_VAL;
                        if (r == 0) {
                                std::vector<double> x(m->nvars, 0.0);
                                double diag[5];
                                acd::SolveStats st;
                                // a short run first (kernel and memory warm-up)
                                r = acd::run_approx(d, hv, x.data(), iterations / 8 + 1, 0.0,
                                                    -HUGE_VAL, 0.0, nullptr, 0, diag, 0.0, st);
                                std::fill(x.begin(), x.end(), 0.0);
                                if (r >= 0)
                                        r = acd::run_approx(d, hv, x.data(), iterations, 0.0,
                                                            -HUGE_VAL, 0.0, nullptr, 0, diag, 0.0,
                                                            st);
                                if (r >= 0)
                                        sec = st.seconds;
                        }
                        d.destroy();
                        if (r < 0)
                                return r;
                        if (sec < best_s) {
                                best_s = sec;
                                best = cap;
                        }
                }
                std::lock_guard<std::mutex> tg(g_tune_mu);
                g_tuned[key] = best;
        }
        if (!(a->lay_ready && a->lay.max_steps == best)) {
                // rebuilt on the next solve with the chosen cap
                a->lay_max_steps = best;
                a->lay_ready = false;
                if (a->dev_ready) {
                        a->dev.destroy();
                        a->dev = acd::DevInstance();
                        a->dev_ready = false;
                }
        }
        if (chosen)
                *chosen = best;
        return 0;
}
