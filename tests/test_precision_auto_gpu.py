"""ACDALM_PRECISION_AUTO: FP32 inner iterations (the mixed form) for an LP
with at least 500,000 nonzeros, the FP64 form below, in alm_solve and in
the server; the solve then meets the same FP64 stop."""
import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu

AUTO = 2
THRESHOLD = 500_000


def _capped(lp, budget):
    b = binding()
    m = b.Matrix(lp)
    a = b.Alm(m, lp)
    a.set_kkt_tolerance(1e-6)
    a.set_precision(AUTO)
    a.set_inner_budget(budget)
    a.solve(1000)
    st = a.stats()
    a.free()
    m.free()
    return st


def test_auto_runs_fp64_below_the_threshold(instances):
    lp = instances.batch_instance(2000, 77)
    assert lp.nnz < THRESHOLD
    st = _capped(lp, 400)
    assert st["precision"] == 0 and st["fp32_inner_iterations"] == 0, st


def test_auto_runs_fp32_iterations_from_the_threshold(instances):
    lp = instances.batch_instance(42000, 78)
    assert lp.nnz >= THRESHOLD
    st = _capped(lp, 400)
    assert st["precision"] == 1 and st["fp32_inner_iterations"] > 0, st


def test_auto_in_the_server_meets_the_fp64_stop(instances):
    b = binding()
    small = instances.batch_instance(1500, 79)
    srv = b.Server(precision=AUTO, kkt_tol=1e-6)
    rid = srv.submit(small)
    got = []
    while not got:
        got = srv.poll(timeout=1.0)
    r, x, lam, st, lat = srv.result(got[0])
    srv.close()
    assert r == 0 and st["precision"] == 0, st
    k = instances.rel_kkt(small, x, lam)
    assert k["rel_kkt"] <= 1.01e-6, k


def test_server_rejects_unknown_precision_modes():
    b = binding()
    with pytest.raises(b.AcdalmError):
        b.Server(precision=3)
