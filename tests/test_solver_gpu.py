"""Device solver parity against the oracle (the reference restated, itself
pinned bit-exact to the reference):

* step sizes (approx.c:135-186) are bit-identical;
* with the reference's rounding (acdalm_set_rounding(1)) APPROX iterates
  follow the oracle's to 1e-9 relative (only reductions sum in another
  order), and with fused multiply-adds to 1e-6;
* the full ALM + APPROX solve reaches the reference's objective within
  1e-6 relative and a relative KKT residual below 1e-6.
"""
import os
import re
import tempfile

import numpy as np
import pytest

from golden_io import GOLDEN, load_lp
from libutil import binding, ragged_lp

pytestmark = pytest.mark.gpu


@pytest.fixture
def exact_rounding():
    L = binding().lib()
    L.acdalm_set_rounding.argtypes = [__import__("ctypes").c_int]
    old = L.acdalm_set_rounding(1)
    yield
    L.acdalm_set_rounding(old)


def _small():
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    return g, load_lp(g, "")


def test_step_sizes_bit_identical(oracle_lib, instances):
    b = binding()
    for seed, (m_, n_, k) in enumerate([(1000, 2000, 5), (77, 300, 3), (5, 4, 2)]):
        lp = instances.small(seed=40 + seed, m=m_, n=n_, per_col=min(k, m_))
        w = np.random.default_rng(seed).uniform(0.5, 3, lp.nrows)
        m = b.Matrix(lp)
        a = b.Approx(m, lp, weight=w)
        beta, v, inv_v = a.step_sizes()
        mo = oracle_lib.matrix(lp, 0)
        ao = oracle_lib.approx(mo, lp, weight=w)
        internals = oracle_lib.internals(ao, lp.nrows, lp.ncols, True)
        pm = a.permuted_matrix().layouts()
        cidx, cridx = pm["cperm"]
        ridx_r = pm["rperm"][1]
        assert v.tobytes() == internals["v"][cridx].tobytes()
        assert inv_v.tobytes() == internals["inv_v"][cridx].tobytes()
        assert (beta == internals["beta"][ridx_r]).all()
        oracle_lib.approx_free(ao)
        oracle_lib.matrix_free(mo)
        a.free()
        m.free()


@pytest.mark.parametrize("mode", ["0", "1", "auto"])
def test_step_sizes_bit_identical_all_slice_kinds(mode, oracle_lib, instances, monkeypatch):
    """v_j = sum_i w_i beta_i A_ij^2 stays bit-identical whether the A'
    slices hold 1 or 4 entries per lane and step (ACDALM_SELL_VEC)."""
    monkeypatch.setenv("ACDALM_SELL_VEC", mode)
    b = binding()
    lp = ragged_lp(instances, 22)
    # transpose so that A' has the ragged rows
    lp = instances.LP(lp.ncols, lp.nrows, lp.cols.copy(), lp.rows.copy(), lp.vals.copy(),
                      np.zeros(lp.ncols), np.zeros(lp.nrows), np.zeros(lp.nrows),
                      np.ones(lp.nrows), np.full(lp.ncols, -np.inf),
                      np.full(lp.ncols, np.inf), "ragged_t", 22)
    w = np.random.default_rng(5).uniform(0.5, 3, lp.nrows)
    m = b.Matrix(lp)
    a = b.Approx(m, lp, weight=w)
    beta, v, inv_v = a.step_sizes()
    mo = oracle_lib.matrix(lp, 0)
    ao = oracle_lib.approx(mo, lp, weight=w)
    internals = oracle_lib.internals(ao, lp.nrows, lp.ncols, True)
    cridx = a.permuted_matrix().layouts()["cperm"][1]
    assert v.tobytes() == internals["v"][cridx].tobytes()
    assert inv_v.tobytes() == internals["inv_v"][cridx].tobytes()
    oracle_lib.approx_free(ao)
    oracle_lib.matrix_free(mo)
    a.free()
    m.free()


@pytest.mark.parametrize("niter", [1, 2, 10, 40])
def test_approx_iterates_follow_oracle(niter, exact_rounding, oracle_lib):
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    mo = oracle_lib.matrix(lp, 0)
    ao = oracle_lib.approx(mo, lp)
    x0 = np.full(lp.ncols, 1.0)
    r1, x1, d1 = a.solve(x0, niter, max_pg=1e-12)
    r2, x2, d2 = oracle_lib.approx_solve(ao, x0, niter, max_pg=1e-12)
    assert r1 == r2
    scale = np.abs(x2).max()
    assert np.abs(x1 - x2).max() <= 1e-9 * scale, np.abs(x1 - x2).max()
    assert np.allclose(d1, d2, rtol=1e-9, atol=1e-12)
    oracle_lib.approx_free(ao)
    oracle_lib.matrix_free(mo)
    a.free()
    m.free()


def test_approx_fused_rounding_close_to_oracle(oracle_lib):
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    mo = oracle_lib.matrix(lp, 0)
    ao = oracle_lib.approx(mo, lp)
    x0 = np.zeros(lp.ncols)
    r1, x1, d1 = a.solve(x0, 25)
    r2, x2, d2 = oracle_lib.approx_solve(ao, x0, 25)
    assert np.abs(x1 - x2).max() <= 1e-6 * np.abs(x2).max()
    assert abs(d1[0] - d2[0]) <= 1e-6 * abs(d2[0])
    oracle_lib.approx_free(ao)
    oracle_lib.matrix_free(mo)
    a.free()
    m.free()


def test_alm_solve_reaches_reference_optimum(instances):
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    with tempfile.TemporaryDirectory() as td:
        log = os.path.join(td, "alm.log")
        r, x, lam, diag = alm.solve(1000, log=log)
        text = open(log).read()
    st = alm.stats()
    ref_obj = float(g["alm.diag"][0])
    assert r == 0
    assert abs(diag[0] - ref_obj) <= 1e-6 * abs(ref_obj), (diag[0], ref_obj)
    k = instances.rel_kkt(lp, x, lam)
    assert k["rel_kkt"] < 1e-6, k
    assert abs(st["rel_kkt"] - k["rel_kkt"]) <= 1e-9 + 1e-3 * k["rel_kkt"]
    # the reference's outer log line format (alm.c:260-285)
    outer = re.findall(r"^ *(\d+): +\S+ +\S+ +\S+ +\S+ +\S+ (-stalled-|\( *\S+\))$", text,
                       re.M)
    assert len(outer) == st["outer_iterations"] >= 1
    # inner lines (approx.c:504-515), possibly after restart markers
    inner = re.findall(r"^(?:\t\t R+)?\t +\d+ +\S+ +\S+ +\S+ +\S+(?: +\S+)?$", text, re.M)
    assert len(inner) >= 2 * len(outer)
    alm.free()
    m.free()


def test_alm_warm_start_and_kkt_stop(instances):
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_kkt_tolerance(1e-6)
    r, x, lam, diag = alm.solve(1000)
    st = alm.stats()
    k = instances.rel_kkt(lp, x, lam)
    assert st["rel_kkt"] <= 1e-6 and k["rel_kkt"] <= 1.01e-6, (st, k)
    r2, x2, lam2, _ = alm.solve(1000, x=x, lam=lam)
    st2 = alm.stats()
    assert st2["inner_iterations"] < st["inner_iterations"]
    alm.free()
    m.free()


def test_inner_budget_caps_iterations():
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_inner_budget(700)
    alm.solve(1000)
    st = alm.stats()
    assert st["inner_iterations"] <= 700
    alm.free()
    m.free()


def test_mpg_follows_oracle(oracle_lib):
    b = binding()
    g, lp = _small()
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    mo = oracle_lib.matrix(lp, 0)
    ao = oracle_lib.approx(mo, lp)
    r1, x1, d1 = a.mpg_solve(np.zeros(lp.ncols), 50)
    r2, x2, d2 = oracle_lib.mpg_solve(ao, np.zeros(lp.ncols), 50)
    assert r1 == r2 == 2
    assert np.abs(x1 - x2).max() <= 1e-6 * np.abs(x2).max()
    assert np.allclose(d1[:3], d2[:3], rtol=1e-6)
    oracle_lib.approx_free(ao)
    oracle_lib.matrix_free(mo)
    a.free()
    m.free()
