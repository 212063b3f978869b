"""Batched solves (one LP per CTA, acdalm_batch_*): every LP of a batch
reaches the oracle's optimum, and each LP's result is the same -- bit for
bit -- whether it is solved alone or in the mix with others."""
import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu


def _lps(instances, count, seed):
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(40), np.log(400), size=count))).astype(int)
    return [instances.batch_instance(int(m), seed * 1000 + i) for i, m in enumerate(sizes)]


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_reaches_oracle_optimum(precision, instances, oracle_lib):
    b = binding()
    lps = _lps(instances, 12, 7 + precision)
    mats = [b.Matrix(lp) for lp in lps]
    alms = [b.Alm(m, lp) for m, lp in zip(mats, lps)]
    for a in alms:
        a.set_kkt_tolerance(1e-6)
        a.set_precision(precision)
    batch = b.Batch(alms)
    ret, xs, lams, diag = batch.solve(1000)
    for i, lp in enumerate(lps):
        assert ret[i] == 0, (i, ret[i])
        k = instances.rel_kkt(lp, xs[i], lams[i])
        assert k["rel_kkt"] <= 1.01e-6, (i, k)
        mo = oracle_lib.matrix(lp)
        ho = oracle_lib.alm(mo, lp)
        _, xo, lo, do, _ = oracle_lib.alm_solve(ho, lp.nrows, lp.ncols)
        ko = instances.rel_kkt(lp, xo, lo)
        scale = abs(ko["objective"]) + 1
        # both within ~1e-6 relative KKT of the same LP optimum
        assert abs(k["objective"] - ko["objective"]) <= 1e-5 * scale, (i, k, ko)
        oracle_lib.alm_free(ho)
        oracle_lib.matrix_free(mo)
    assert batch.seconds() > 0
    batch.free()
    for a in alms:
        a.free()
    for m in mats:
        m.free()


def test_same_alone_and_in_the_mix(instances):
    b = binding()
    lps = _lps(instances, 9, 21)
    mats = [b.Matrix(lp) for lp in lps]

    def solve(group):
        alms = [b.Alm(mats[i], lps[i]) for i in group]
        for a in alms:
            a.set_kkt_tolerance(1e-6)
            a.set_precision(1)
        batch = b.Batch(alms)
        ret, xs, lams, _ = batch.solve(1000)
        batch.free()
        for a in alms:
            a.free()
        return dict(zip(group, zip(xs, lams)))

    mixed = solve(list(range(len(lps))))
    for i in (0, 4, 8):
        alone = solve([i])
        assert alone[i][0].tobytes() == mixed[i][0].tobytes(), i
        assert alone[i][1].tobytes() == mixed[i][1].tobytes(), i
    for m in mats:
        m.free()
