"""Input checks of the solve entry points, on the host (no GPU needed: they
run before any device work).  The reference asserts that its iterates stay
finite (approx/step_project.inc:90, :577); a NaN or an infinity in the
problem data makes them non-finite from the first step, so the library
refuses such inputs with ACDALM_ENONFINITE and names the offending entry."""
import ctypes

import numpy as np
import pytest

from libutil import binding

ENONFINITE = -5


def _alm(b, lp):
    m = b.Matrix(lp)
    return m, b.Alm(m, lp)


@pytest.mark.parametrize("field,value", [("linear", np.nan), ("rhs", np.nan),
                                         ("rhs", np.inf), ("linear", -np.inf),
                                         ("lower", np.nan), ("upper", np.nan)])
def test_alm_solve_refuses_non_finite_data(field, value, instances):
    b = binding()
    L = b.lib()
    lp = instances.small(seed=8, m=30, n=60, per_col=3)
    getattr(lp, field)[7] = value
    m, alm = _alm(b, lp)
    x = np.zeros(lp.ncols)
    lam = np.zeros(lp.nrows)
    r = L.alm_solve(alm.h, 10, x, lp.ncols, lam, lp.nrows, None, np.zeros(3), None)
    assert r == ENONFINITE
    msg = L.acdalm_last_error().decode()
    assert field in msg and "[7]" in msg, msg
    alm.free()
    m.free()


def test_alm_solve_refuses_non_finite_start(instances):
    b = binding()
    L = b.lib()
    lp = instances.small(seed=9, m=30, n=60, per_col=3)
    m, alm = _alm(b, lp)
    x = np.zeros(lp.ncols)
    lam = np.zeros(lp.nrows)
    lam[3] = np.nan
    r = L.alm_solve(alm.h, 10, x, lp.ncols, lam, lp.nrows, None, np.zeros(3), None)
    assert r == ENONFINITE and b"lambda[3]" in L.acdalm_last_error()
    alm.free()
    m.free()


def test_infinite_bounds_are_accepted_as_bounds(instances):
    """Infinite box bounds are legal (alm_make's defaults are +-inf): the
    check lets them through, and the call goes on to the device (which, on a
    machine without one, reports ACDALM_ENODEV; with one, solves)."""
    b = binding()
    L = b.lib()
    lp = instances.small(seed=10, m=30, n=60, per_col=3)
    lp.upper[:] = np.inf
    m, alm = _alm(b, lp)
    r = L.alm_solve(alm.h, 1, np.zeros(lp.ncols), lp.ncols, np.zeros(lp.nrows), lp.nrows,
                    None, np.zeros(3), None)
    assert r != ENONFINITE
    alm.free()
    m.free()


def test_approx_solve_refuses_non_finite_weight(instances):
    b = binding()
    L = b.lib()
    lp = instances.small(seed=11, m=30, n=60, per_col=3)
    w = np.ones(lp.nrows)
    w[2] = np.nan
    m = b.Matrix(lp)
    a = b.Approx(m, lp, weight=w)
    x = np.zeros(lp.ncols)
    r = L.approx_solve(x, lp.ncols, a.h, 10, 0.0, -np.inf, 0.0, None, 0, np.zeros(5), 0.0,
                       None)
    assert r == ENONFINITE and b"weight[2]" in L.acdalm_last_error()
    a.free()
    m.free()
