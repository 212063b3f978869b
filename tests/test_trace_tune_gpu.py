"""Tracing and autotuning of the whole-GPU solve.

alm_set_trace / alm_trace_copy: every CTA stamps each traced team reduction
three times, in order -- entering it, after its block reduction, leaving it
-- and a reduction starts only after the previous one ended in that CTA; no
CTA leaves a reduction before every CTA has finished its block reduction
(the reduction is a barrier).  acdalm_autotune: picks one of its candidate
layouts, and the solve keeps its answer."""
import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu


def test_trace_stamps_are_ordered(instances):
    b = binding()
    lp = instances.small(seed=41, m=500, n=1000, per_col=5)
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_inner_budget(200)
    alm.set_trace(11, 64)
    r, x, lam, _ = alm.solve(1000)
    t = alm.trace().astype(np.int64)
    assert t.shape[0] == 64 and t.shape[1] >= 1 and t.shape[2] == 3
    assert (t > 0).all()
    assert (t[:, :, 0] <= t[:, :, 1]).all() and (t[:, :, 1] <= t[:, :, 2]).all()
    assert (t[1:, :, 0] >= t[:-1, :, 2]).all()
    # a barrier: every CTA leaves after the last CTA's block reduction (the
    # timer is global; 500 ns of slack for its resolution)
    assert (t[:, :, 2].min(axis=1) + 500 >= t[:, :, 1].max(axis=1)).all()
    # tracing does not change the answer (a fresh instance: the ALM weights
    # persist across solves of one instance)
    alm2 = b.Alm(m, lp)
    alm2.set_inner_budget(200)
    r2, x2, lam2, _ = alm2.solve(1000)
    assert x.tobytes() == x2.tobytes() and lam.tobytes() == lam2.tobytes()
    alm2.free()
    alm.free()
    m.free()


def test_autotune_picks_a_candidate_and_keeps_the_answer(instances):
    """acdalm_autotune times the candidate layouts and keeps one; the solve
    that follows reaches the same stop, and a second instance of the same
    size class reuses the choice."""
    b = binding()
    lp = instances.small(seed=42, m=800, n=1600, per_col=5)
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_kkt_tolerance(1e-6)
    chosen = alm.autotune(100)
    assert chosen in (0, 4, 8, 12, 16)
    r, x, lam, _ = alm.solve(1000)
    assert r == 0 and instances.rel_kkt(lp, x, lam)["rel_kkt"] <= 1.01e-6
    alm2 = b.Alm(m, lp)
    assert alm2.autotune(100) == chosen
    alm2.free()
    alm.free()
    m.free()
