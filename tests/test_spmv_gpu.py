"""Device SpMV parity (spmv.c:159-233, spmv_block.c:160-320): the SELL and
block variants add each row in the reference's order with the reference's
rounding, so they match the oracle (the reference restated) bit for bit;
the CSR and fused SELL variants re-associate and are held to 1e-12
relative."""
import numpy as np
import pytest

from libutil import binding, ragged_lp

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (5, 3, 2), (33, 17, 4), (257, 513, 5), (1000, 2000, 5),
          (4097, 1000, 9)]


def _lp(instances, m, n, k, seed=0):
    lp = instances.small(seed=seed + m * 7 + n, m=m, n=n, per_col=min(k, m))
    return lp


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_multiply_matches_oracle(shape, variant, instances, oracle_lib):
    b = binding()
    L = b.lib()
    lp = _lp(instances, *shape)
    m = b.Matrix(lp)
    mo = oracle_lib.matrix(lp, 0)
    rng = np.random.default_rng(1)
    old = L.acdalm_spmv_variant(variant)
    try:
        for t in (False, True):
            x = rng.uniform(-1, 1, lp.nrows if t else lp.ncols)
            got = m.multiply(x, transpose=t)
            want = oracle_lib.multiply(mo, x, t)
            if variant in (0, 1):
                assert got.tobytes() == want.tobytes(), (shape, variant, t)
            else:
                scale = np.abs(want).max(initial=0) + 1
                assert np.abs(got - want).max(initial=0) <= 1e-12 * scale
            x2 = rng.uniform(-1, 1, x.shape[0])
            y0, y1 = m.multiply_2(x, x2, transpose=t)
            w1 = oracle_lib.multiply(mo, x2, t)
            if variant in (0, 1):
                assert y0.tobytes() == want.tobytes() and y1.tobytes() == w1.tobytes()
            else:
                assert np.allclose(y0, want, rtol=0, atol=1e-12 * (np.abs(want).max(initial=0) + 1))
                assert np.allclose(y1, w1, rtol=0, atol=1e-12 * (np.abs(w1).max(initial=0) + 1))
    finally:
        L.acdalm_spmv_variant(old)
    oracle_lib.matrix_free(mo)
    m.free()


def test_empty_rows_and_columns(instances, oracle_lib):
    """Rows and columns without entries produce exact zeros."""
    b = binding()
    lp = instances.small(seed=11, m=64, n=40, per_col=1)
    keep = lp.cols % 3 != 0
    lp.rows, lp.cols, lp.vals = lp.rows[keep], lp.cols[keep], lp.vals[keep]
    m = b.Matrix(lp)
    mo = oracle_lib.matrix(lp, 0)
    for t in (False, True):
        x = np.linspace(-1, 1, lp.nrows if t else lp.ncols)
        assert m.multiply(x, t).tobytes() == oracle_lib.multiply(mo, x, t).tobytes()
    oracle_lib.matrix_free(mo)
    m.free()


def test_device_f32_variants(instances):
    """FP32 device products (values rounded once) stay within FP32
    accumulation error of the FP64 product."""
    import torch
    b = binding()
    L = b.lib()
    lp = instances.small(seed=12, m=3000, n=6000, per_col=6)
    m = b.Matrix(lp)
    x = np.random.default_rng(2).uniform(-1, 1, lp.ncols)
    want = lp.matvec(x)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    for variant in (0, 2):
        yd = torch.zeros(lp.nrows, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        assert L.acdalm_spmv_device_f32(m.h, variant, 0, xd.data_ptr(), yd.data_ptr(),
                                        s) == 0
        torch.cuda.synchronize()
        got = yd.double().cpu().numpy()
        assert np.abs(got - want).max() <= 1e-5 * (np.abs(want).max() + 1)
    m.free()


@pytest.mark.parametrize("mode", ["0", "1", "auto"])
def test_sell_slice_kinds_match_oracle(mode, instances, oracle_lib, monkeypatch):
    """Scalar-only, vector-only and mixed SELL layouts (ACDALM_SELL_VEC) all
    reproduce the reference's row sums bit for bit, for every lane count
    (rows of 0..700 entries), one and two right-hand sides."""
    monkeypatch.setenv("ACDALM_SELL_VEC", mode)
    b = binding()
    L = b.lib()
    lp = ragged_lp(instances, 21)
    m = b.Matrix(lp)
    mo = oracle_lib.matrix(lp, 0)
    rng = np.random.default_rng(3)
    old = L.acdalm_spmv_variant(0)
    try:
        for t in (False, True):
            x = rng.uniform(-1, 1, lp.nrows if t else lp.ncols)
            x2 = rng.uniform(-1, 1, x.shape[0])
            want = oracle_lib.multiply(mo, x, t)
            assert m.multiply(x, transpose=t).tobytes() == want.tobytes(), t
            y0, y1 = m.multiply_2(x, x2, transpose=t)
            assert y0.tobytes() == want.tobytes()
            assert y1.tobytes() == oracle_lib.multiply(mo, x2, t).tobytes()
    finally:
        L.acdalm_spmv_variant(old)
    oracle_lib.matrix_free(mo)
    m.free()


def test_fp32_long_rows_error_bound(instances):
    """FP32 row sums on rows of 0..700 entries (every lane count).  The SELL
    layout never gives one lane a chain of more than 64 products (rows over
    16 entries spread over 4, 16 or 32 lanes, 4 entries per lane and step in
    vector slices), and rows wider than 256 entries combine their lanes'
    partial sums in FP64, so the accumulation error of a row stays within

        |y32_i - y_i| <= (min(len_i, 64) + 4) * 2^-24 * sum_k |a_ik x_k|

    against the exact product of the same FP32-rounded values and vector,
    where one FP32 chain over a 700-entry row could be off by 704 units.
    The CSR kernel is held to the plain (len_i + 4) bound.  Both are also
    within 4 * 2^-24 * sum |a x| of that bound from the FP64 product of the
    unrounded data."""
    import torch
    b = binding()
    L = b.lib()
    lp = ragged_lp(instances, 24)
    m = b.Matrix(lp)
    rng = np.random.default_rng(6)
    u32 = 2.0 ** -24
    lens = np.bincount(lp.rows, minlength=lp.nrows)
    assert lens.max() > 600
    x = rng.uniform(-1, 1, lp.ncols)
    x32 = x.astype(np.float32)
    a32 = lp.vals.astype(np.float32).astype(np.float64)
    exact = np.bincount(lp.rows, weights=a32 * x32.astype(np.float64)[lp.cols],
                        minlength=lp.nrows)
    mag = np.bincount(lp.rows, weights=np.abs(a32 * x32.astype(np.float64)[lp.cols]),
                      minlength=lp.nrows)
    for variant, chain in ((0, np.minimum(lens, 64)), (2, lens)):
        bound = (chain + 4) * u32 * mag
        xd = torch.tensor(x32, device="cuda")
        yd = torch.zeros(lp.nrows, dtype=torch.float32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        assert L.acdalm_spmv_device_f32(m.h, variant, 0, xd.data_ptr(), yd.data_ptr(), s) == 0
        torch.cuda.synchronize()
        got = yd.double().cpu().numpy()
        err = np.abs(got - exact)
        assert (err <= bound).all(), (variant, np.max(err / np.maximum(bound, 1e-300)))
        full = lp.matvec(x)
        assert (np.abs(got - full) <= bound + 4 * u32 * mag).all(), variant
    m.free()


def test_mixed_solve_on_long_rows_reaches_oracle_optimum(instances, oracle_lib):
    """The mixed-precision solve (FP32 inner iterations) on an LP whose rows
    have up to 700 entries meets the FP64 stop and the oracle's optimum."""
    b = binding()
    lp = ragged_lp(instances, 25)
    m = b.Matrix(lp)
    alm = b.Alm(m, lp)
    alm.set_kkt_tolerance(1e-6)
    alm.set_precision(1)
    r, x, lam, _ = alm.solve(1000)
    st = alm.stats()
    assert r == 0 and st["fp32_inner_iterations"] > 0, st
    k = instances.rel_kkt(lp, x, lam)
    assert k["rel_kkt"] <= 1.01e-6, k
    mo = oracle_lib.matrix(lp)
    ho = oracle_lib.alm(mo, lp)
    _, xo, lo, _, _ = oracle_lib.alm_solve(ho, lp.nrows, lp.ncols)
    ko = instances.rel_kkt(lp, xo, lo)
    assert abs(k["objective"] - ko["objective"]) <= 1e-5 * (abs(ko["objective"]) + 1), (k, ko)
    oracle_lib.alm_free(ho)
    oracle_lib.matrix_free(mo)
    alm.free()
    m.free()
