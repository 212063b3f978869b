"""The covering LP (A x >= 1 with 0/1 coefficients, slack columns making
it [A -I][x; s] = 1, multipliers >= 0), reduced to m = 5,000 rows and
20,000 structural columns, solved end to end on the whole GPU in both
precision forms against the reference's own solve of the same LP to
relative KKT <= 1e-6 (tests/golden/covering_kkt.npz, made by
tests/golden/make_kkt_golden.py: alm.c:289-322 over approx/approx.c:576-708)."""
import os

import numpy as np
import pytest

from golden_io import GOLDEN
from libutil import binding

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_covering_lp_matches_reference(precision, instances):
    g = np.load(os.path.join(GOLDEN, "covering_kkt.npz"))
    lp = instances.covering(m=5000, n=20000)
    assert lp.sha256() == str(g["instance_sha256"])
    b = binding()
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_kkt_tolerance(1e-6)
    alm.set_precision(precision)
    r, x, lam, _ = alm.solve(1000)
    st = alm.stats()
    assert r == 0 and st["rel_kkt"] <= 1e-6, st
    k = instances.rel_kkt(lp, x, lam)
    assert k["rel_kkt"] <= 1.01e-6, k
    # the slacks are nonnegative and the covering rows hold to the tolerance
    assert (x >= 0).all()
    ax = lp.matvec(x)
    assert np.abs(ax - lp.rhs).max() <= 1e-3
    ref = float(g["objective"])
    assert abs(k["objective"] - ref) <= 1e-6 * abs(ref), (k["objective"], ref)
    if precision:
        assert st["fp32_inner_iterations"] > 0
    alm.free()
    m.free()
