"""Failure paths of the device solve, in forms that never fault or hang a
GPU: the whole-solve time limit (ACDALM_SOLVE_TIMEOUT) runs out on a small
LP, every thread of the team stops at the same check, the call returns
ACDALM_ETIMELIMIT with a message naming the limit, and the next solve on
the same instance succeeds."""
import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu

ETIMELIMIT = -7


def test_alm_solve_time_limit_then_recovers(instances, monkeypatch):
    b = binding()
    L = b.lib()
    lp = instances.small(seed=31, m=400, n=800, per_col=5)
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_kkt_tolerance(1e-6)
    # 100 microseconds: the first check, after 100 inner iterations, is past it
    monkeypatch.setenv("ACDALM_SOLVE_TIMEOUT", "1e-4")
    x = np.zeros(lp.ncols)
    lam = np.zeros(lp.nrows)
    r = L.alm_solve(alm.h, 1000, x, lp.ncols, lam, lp.nrows, None, np.zeros(3), None)
    assert r == ETIMELIMIT
    assert b"time limit" in L.acdalm_last_error()
    assert alm.stats()["status"] == ETIMELIMIT
    monkeypatch.delenv("ACDALM_SOLVE_TIMEOUT")
    r, x, lam, _ = alm.solve(1000)
    assert r == 0
    assert instances.rel_kkt(lp, x, lam)["rel_kkt"] <= 1.01e-6
    alm.free()
    m.free()


def test_approx_solve_time_limit_then_recovers(instances, monkeypatch):
    b = binding()
    L = b.lib()
    lp = instances.small(seed=32, m=300, n=600, per_col=5)
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    monkeypatch.setenv("ACDALM_SOLVE_TIMEOUT", "1e-4")
    x = np.zeros(lp.ncols)
    r = L.approx_solve(x, lp.ncols, a.h, 5000, 0.0, -np.inf, 0.0, None, 0, np.zeros(5), 0.0,
                       None)
    assert r == ETIMELIMIT
    monkeypatch.delenv("ACDALM_SOLVE_TIMEOUT")
    r, x, d = a.solve(np.zeros(lp.ncols), 500)
    assert r == 0 and d[4] == 501
    a.free()
    m.free()


def test_batch_time_limit_is_per_lp(instances, monkeypatch):
    """In a batch (one CTA per LP) the limit stops each LP by itself; the
    batch reports the code and a following batch solves them all."""
    b = binding()
    lps = [instances.batch_instance(int(mm), 600 + i) for i, mm in enumerate((120, 300, 500))]
    mats = [b.Matrix(lp) for lp in lps]
    alms = [b.Alm(mm, lp) for mm, lp in zip(mats, lps)]
    for a in alms:
        a.set_kkt_tolerance(1e-6)
    monkeypatch.setenv("ACDALM_SOLVE_TIMEOUT", "1e-4")
    batch = b.Batch(alms)
    with pytest.raises(b.AcdalmError):
        batch.solve(1000)
    monkeypatch.delenv("ACDALM_SOLVE_TIMEOUT")
    batch.free()
    batch = b.Batch(alms)
    ret, xs, lams, _ = batch.solve(1000)
    assert (np.asarray(ret) == 0).all()
    batch.free()
    for a in alms:
        a.free()
    for mm in mats:
        mm.free()
