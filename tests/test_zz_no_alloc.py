"""approx_solve_static, the allocation-free APPROX entry point, called through
the C ABI.

Who needs it: a caller whose framework has already handed the GPU's memory
to its own caching allocator (a cudaMalloc beside it fails or fragments the
pool), or a latency-bound loop that cannot take cudaMalloc's device-wide
synchronisation.  The entry point keeps its scratch in one fixed device
array inside the library instead of allocating.

Its answers must be those of approx_solve on the same instance, bit for
bit (same kernel, same grid, so the same reduction order): on two calls in
a row, after a call that stopped at once (its reduction lines are left
with low epoch tags the next launch must not mistake for its own), and
alternating between two instances of different sizes that share the array.

This file sorts last, so a failure here leaves every other test's result
in place."""
import ctypes

import numpy as np
import pytest

from libutil import binding

pytestmark = pytest.mark.gpu

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


def _entry(L):
    f = L.approx_solve_static
    f.restype = ctypes.c_int
    f.argtypes = [_vp, _sz, _vp, _sz, ctypes.c_double, ctypes.c_double,
                  ctypes.c_double, _vp, ctypes.c_double, _vp]
    return f


def _static(L, solve_static, a, lp, x0, niter):
    """One approx_solve_static call; returns (reason, x, diagnosis)."""
    import torch
    xd = torch.tensor(x0, dtype=torch.float64, device="cuda")
    diag = np.zeros(5)
    stream = torch.cuda.current_stream().cuda_stream
    r = solve_static(xd.data_ptr(), lp.ncols, a.h, niter, 1e-9, -np.inf, 0.0,
                     diag.ctypes.data_as(_vp), 0.0, stream)
    assert r >= 0, L.acdalm_last_error()
    return r, xd.cpu().numpy(), diag


def _same(got, want, what):
    r, x, d = got
    r0, x0, d0 = want
    assert r == r0, what
    assert x.tobytes() == x0.tobytes(), (what, np.abs(x - x0).max())
    assert d.tobytes() == d0.tobytes(), (what, d, d0)


def test_static_solve_matches_approx_solve(instances):
    b = binding()
    L = b.lib()
    solve_static = _entry(L)
    lp = instances.small(seed=21, m=700, n=1500, per_col=5)
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    x0 = np.random.default_rng(3).uniform(0, 10, lp.ncols)
    # approx_solve creates the instance's device copy and gives the answer
    want = a.solve(x0, 400, max_pg=1e-9)
    for call in range(2):
        _same(_static(L, solve_static, a, lp, x0, 400), want, f"call {call}")
    a.free()
    m.free()


def test_static_solve_after_a_call_that_stopped_at_once(instances):
    b = binding()
    L = b.lib()
    solve_static = _entry(L)
    lp = instances.small(seed=23, m=600, n=1300, per_col=5)
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    x0 = np.random.default_rng(4).uniform(0, 10, lp.ncols)
    want = a.solve(x0, 300, max_pg=1e-9)
    for _ in range(2):
        _static(L, solve_static, a, lp, x0, 0)
        _same(_static(L, solve_static, a, lp, x0, 300), want, "after niter = 0")
    a.free()
    m.free()


def test_static_solve_alternating_instances(instances):
    b = binding()
    L = b.lib()
    solve_static = _entry(L)
    lps = [instances.small(seed=25, m=500, n=1000, per_col=5),
           instances.small(seed=26, m=1800, n=4000, per_col=6)]
    mats = [b.Matrix(lp) for lp in lps]
    aps = [b.Approx(mm, lp) for mm, lp in zip(mats, lps)]
    x0s = [np.random.default_rng(5 + i).uniform(0, 10, lp.ncols) for i, lp in enumerate(lps)]
    wants = [a.solve(x0, 250, max_pg=1e-9) for a, x0 in zip(aps, x0s)]
    for turn in range(4):
        i = turn % 2
        _same(_static(L, solve_static, aps[i], lps[i], x0s[i], 250), wants[i],
              f"turn {turn}, instance {i}")
    for a in aps:
        a.free()
    for mm in mats:
        mm.free()


def test_static_solve_rejects_instances_over_its_limit(instances):
    b = binding()
    L = b.lib()
    solve_static = _entry(L)
    n = 400_000  # 12 n alone exceeds the 4.17 million doubles the array holds
    lp = instances.LP(nrows=1, ncols=n, rows=np.zeros(n, np.uint32),
                      cols=np.arange(n, dtype=np.uint32), vals=np.ones(n),
                      rhs=np.ones(1), linear=np.zeros(n), lower=np.zeros(n),
                      upper=np.ones(n), lambda_lower=np.full(1, -np.inf),
                      lambda_upper=np.full(1, np.inf))
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    import torch
    xd = torch.zeros(n, dtype=torch.float64, device="cuda")
    r = solve_static(xd.data_ptr(), n, a.h, 10, 0.0, -np.inf, 0.0, None, 0.0, None)
    assert r == -4  # ACDALM_EINVAL
    assert b"scratch" in L.acdalm_last_error()
    a.free()
    m.free()
