"""The LP server (acdalm_server_*): requests submitted while others run are
admitted and solved beside them; every LP reaches a relative KKT residual
<= 1e-6, and its result is bit-identical whether it was solved alone (a
server holding only it) or in the mix of a busy server."""
import time

import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu


def _lps(instances, count, seed):
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(50), np.log(600), size=count))).astype(int)
    return [instances.batch_instance(int(m), seed * 7919 + i) for i, m in enumerate(sizes)]


def _serve(b, lps, gap=0.0, **kw):
    srv = b.Server(**kw)
    ids = []
    for lp in lps:
        ids.append(srv.submit(lp))
        if gap:
            time.sleep(gap)
    out = {}
    deadline = time.time() + 300
    while len(out) < len(ids) and time.time() < deadline:
        for rid in srv.poll(timeout=0.5):
            out[rid] = srv.result(rid)
    srv.close()
    assert len(out) == len(ids)
    return [out[i] for i in ids]


def test_server_solves_every_request(instances):
    b = binding()
    lps = _lps(instances, 16, 3)
    res = _serve(b, lps, gap=0.002, max_inflight=6)
    for lp, (r, x, lam, st, lat) in zip(lps, res):
        assert r == 0, st
        k = instances.rel_kkt(lp, x, lam)
        assert k["rel_kkt"] <= 1.01e-6, k
        assert st["rel_kkt"] <= 1e-6
        assert lat > 0


def test_same_alone_and_in_the_mix(instances):
    b = binding()
    lps = _lps(instances, 12, 5)
    mixed = _serve(b, lps, max_inflight=12)
    for i in (0, 5, 11):
        alone = _serve(b, [lps[i]], max_inflight=1)[0]
        assert alone[1].tobytes() == mixed[i][1].tobytes(), i
        assert alone[2].tobytes() == mixed[i][2].tobytes(), i


def test_budget_admits_one_at_a_time(instances):
    """A budget that fits one instance still serves them all, in order."""
    b = binding()
    lps = _lps(instances, 4, 9)
    res = _serve(b, lps, device_budget=24 << 20, max_inflight=8)
    assert all(r[0] == 0 for r in res)


def test_large_lp_runs_on_a_cluster(instances):
    """An LP with more than 150k nonzeros is solved by a thread-block cluster
    of CTAs; it reaches the KKT target and repeats bit for bit."""
    b = binding()
    lp = instances.batch_instance(12600, 77)  # 151,200 nonzeros: 4 CTAs
    assert lp.nnz > 150000
    first = _serve(b, [lp], max_inflight=4, precision=0)[0]
    again = _serve(b, [lp, _lps(instances, 1, 99)[0]], max_inflight=4, precision=0)[0]
    assert first[0] == 0
    k = instances.rel_kkt(lp, first[1], first[2])
    assert k["rel_kkt"] <= 1.01e-6, k
    assert first[1].tobytes() == again[1].tobytes()


def _oracle_objective(oracle_lib, instances, lp, threads=1):
    mo = oracle_lib.matrix(lp)
    ho = oracle_lib.alm(mo, lp)
    _, xo, lo, _, _ = oracle_lib.alm_solve(ho, lp.nrows, lp.ncols, threads=threads)
    oracle_lib.alm_free(ho)
    oracle_lib.matrix_free(mo)
    return instances.rel_kkt(lp, xo, lo)["objective"]


def test_served_lps_reach_oracle_optimum(instances, oracle_lib):
    """Each LP served in a busy mix (mixed precision, the server's default)
    reaches the optimum the oracle's own ALM solve finds, within what two
    points that each meet a 1e-6 relative KKT tolerance can differ by."""
    b = binding()
    lps = _lps(instances, 8, 13)
    res = _serve(b, lps, max_inflight=8)
    for lp, (r, x, lam, st, lat) in zip(lps, res):
        assert r == 0, st
        k = instances.rel_kkt(lp, x, lam)
        assert k["rel_kkt"] <= 1.01e-6, k
        obj = _oracle_objective(oracle_lib, instances, lp)
        assert abs(k["objective"] - obj) <= 1e-5 * (abs(obj) + 1), (k, obj)


def test_large_lp_cluster_mixed_precision(instances, oracle_lib):
    """The cluster team in the mixed form: FP32 inner iterations with the
    float-float partials combined across the cluster's CTAs through
    distributed shared memory, then the FP64 refinement.  It meets the FP64
    stop, reaches the oracle's optimum and repeats bit for bit."""
    b = binding()
    lp = instances.batch_instance(12600, 78)  # 151,200 nonzeros: 4 CTAs
    assert lp.nnz > 150000
    first = _serve(b, [lp], max_inflight=4, precision=1)[0]
    again = _serve(b, [lp, _lps(instances, 1, 98)[0]], max_inflight=4, precision=1)[0]
    r, x, lam, st, _ = first
    assert r == 0, st
    assert st["precision"] == 1 and st["fp32_inner_iterations"] > 0, st
    k = instances.rel_kkt(lp, x, lam)
    assert k["rel_kkt"] <= 1.01e-6, k
    assert x.tobytes() == again[1].tobytes()
    obj = _oracle_objective(oracle_lib, instances, lp, threads=8)
    assert abs(k["objective"] - obj) <= 1e-5 * (abs(obj) + 1), (k, obj)


def test_server_inner_budget_caps_each_request(instances):
    """acdalm_server_set_inner_budget caps every request built after it:
    a one-CTA LP and a cluster LP each stop at the cap (alm_solve's 1, the
    iteration limit) instead of solving to the tolerance."""
    b = binding()
    small = instances.batch_instance(400, 91)
    large = instances.batch_instance(20000, 92)  # 240k nonzeros: a cluster
    srv = b.Server(precision=0, kkt_tol=1e-6)
    srv.set_inner_budget(150)
    ids = [srv.submit(small), srv.submit(large)]
    out = {}
    deadline = time.time() + 120
    while len(out) < 2 and time.time() < deadline:
        for rid in srv.poll(timeout=0.5):
            out[rid] = srv.result(rid)
    srv.close()
    assert len(out) == 2
    for rid in ids:
        r, x, lam, st, lat = out[rid]
        assert r == 1, (r, st)
        assert 0 < st["inner_iterations"] <= 150, st
