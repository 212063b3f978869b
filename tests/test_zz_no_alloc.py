"""approx_solve_static, the allocation-free APPROX entry point, called through
the C ABI: its output must match approx_solve's on the same instance, on two
calls in a row (the fixed scratch array keeps the previous call's contents,
which must not leak into the next).

Callers that cannot call cudaMalloc at solve time -- code running under CUDA
graph capture, frameworks whose allocator owns the device memory -- use this
entry point; this file runs last so a failure here leaves every other test's
result intact."""
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


def test_static_solve_matches_approx_solve(instances):
    import torch
    b = binding()
    L = b.lib()
    solve_static = _entry(L)
    lp = instances.small(seed=21, m=700, n=1500, per_col=5)
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    x0 = np.random.default_rng(3).uniform(0, 10, lp.ncols)
    # approx_solve creates the instance's device copy and gives the answer
    r_ref, x_ref, d_ref = a.solve(x0, 400, max_pg=1e-9)
    for call in range(2):
        xd = torch.tensor(x0, dtype=torch.float64, device="cuda")
        diag = np.zeros(5)
        stream = torch.cuda.current_stream().cuda_stream
        r = solve_static(xd.data_ptr(), lp.ncols, a.h, 400, 1e-9, -np.inf, 0.0,
                         diag.ctypes.data_as(_vp), 0.0, stream)
        assert r >= 0, L.acdalm_last_error()
        x = xd.cpu().numpy()
        assert r == r_ref, call
        scale = np.abs(x_ref).max()
        assert np.abs(x - x_ref).max() <= 1e-12 * scale, (call, np.abs(x - x_ref).max())
        assert np.allclose(diag, d_ref, rtol=1e-12, atol=0), (call, diag, d_ref)
    a.free()
    m.free()


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
