"""The C-ABI boundary on CPU: libacdalm.so loads, exports every function the
headers in include/ declare, and its host-only entry points work without a
GPU (the solver entry points report ACDALM_ENODEV instead of computing)."""
import ctypes
import subprocess

import numpy as np
import pytest

from libutil import binding, header_functions


def test_library_exports_every_declared_symbol():
    b = binding()
    names = header_functions()
    assert {"alm_solve", "approx_solve", "sparse_matrix_multiply",
            "thread_pool_map_reduce", "acdalm_last_error"} <= names
    out = subprocess.run(["nm", "-D", "--defined-only", b.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = sorted(names - exported)
    assert not missing, missing


def test_reference_signatures_are_c_abi():
    """Unmangled names: the reference's callers link against them as C."""
    b = binding()
    L = ctypes.CDLL(b.LIB_PATH)
    for name in ("sparse_matrix_make", "sparse_matrix_multiply_2", "approx_make",
                 "approx_update", "mpg_solve", "cd_solve", "alm_make", "alm_read",
                 "thread_pool_init", "thread_pool_for"):
        assert hasattr(L, name), name


def test_thread_pool_semantics():
    """thread_pool_for covers [from, end) once with granularity-aligned
    chunks; map_reduce sums (thread_pool.c:304-401)."""
    b = binding()
    L = b.lib()
    FN = ctypes.CFUNCTYPE(None, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                          ctypes.c_uint)
    MAP = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_size_t, ctypes.c_size_t,
                           ctypes.c_void_p, ctypes.c_uint)
    L.thread_pool_for.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                  ctypes.c_size_t, FN, ctypes.c_void_p]
    L.thread_pool_map_reduce.restype = ctypes.c_double
    L.thread_pool_map_reduce.argtypes = [ctypes.c_void_p, ctypes.c_size_t,
                                         ctypes.c_size_t, ctypes.c_size_t, MAP,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
    for nthreads in (0, 1, 4):
        pool = L.thread_pool_init(nthreads) if nthreads else None
        seen = np.zeros(1000, np.int64)
        chunks = []

        def body(b_, e_, info, wid):
            seen[b_:e_] += 1
            chunks.append((b_, e_))
        cb = FN(body)
        L.thread_pool_for(pool, 0, 1000, 16, cb, None)
        assert (seen == 1).all()
        assert all((e_ - b_) % 16 == 0 or e_ == 1000 for b_, e_ in chunks)
        total = L.thread_pool_map_reduce(pool, 0, 1000, 8,
                                         MAP(lambda b_, e_, i, w: float(sum(range(b_, e_)))),
                                         None, 0, 0.0)
        assert total == 1000 * 999 / 2
        mx = L.thread_pool_map_reduce(pool, 0, 1000, 8,
                                      MAP(lambda b_, e_, i, w: float(e_ - 1)), None, 1,
                                      -np.inf)
        assert mx == 999
        if pool:
            assert L.thread_pool_count(pool) == nthreads
            L.thread_pool_free(pool)


def test_bad_arguments_are_rejected(instances):
    b = binding()
    lp = instances.small(seed=3, m=20, n=30, per_col=3)
    bad = lp.rows.copy()
    bad[0] = lp.nrows  # out of range
    L = b.lib()
    h = L.sparse_matrix_make(lp.ncols, lp.nrows, lp.nnz, bad, lp.cols.astype(np.uint32),
                             lp.vals, 0)
    assert not h
    m = b.Matrix(lp)
    with pytest.raises(b.AcdalmError):
        m.multiply(np.zeros(lp.ncols + 1))
    m.free()


def test_spmv_variant_selector_range():
    """acdalm_spmv_variant accepts the four variants and ignores anything
    else, returning the previous selection (host-only, no GPU needed)."""
    b = binding()
    L = b.lib()
    old = L.acdalm_spmv_variant(b.SPMV_SELL_FMA)
    try:
        assert L.acdalm_spmv_variant(b.SPMV_CSR) == b.SPMV_SELL_FMA
        assert L.acdalm_spmv_variant(4) == b.SPMV_CSR
        assert L.acdalm_spmv_variant(-1) == b.SPMV_CSR
        assert L.acdalm_spmv_variant(b.SPMV_SELL) == b.SPMV_CSR
    finally:
        L.acdalm_spmv_variant(old)


def test_sell_copy_rejects_short_buffers(instances):
    """acdalm_sell_copy reports its sizes, then refuses buffers smaller
    than those sizes instead of writing past them."""
    b = binding()
    L = b.lib()
    lp = instances.small(seed=6, m=40, n=70, per_col=3)
    m = b.Matrix(lp)
    ns, ne = ctypes.c_size_t(), ctypes.c_size_t()
    assert L.acdalm_sell_copy(m.h, 0, ctypes.byref(ns), ctypes.byref(ne),
                              None, None, None, None, None) == 0
    assert ns.value > 0 and ne.value >= lp.nnz and ne.value % 32 == 0
    short = ctypes.c_size_t(ne.value - 1)
    bufs = [np.zeros(ns.value + 1, np.int64), np.zeros(ns.value, np.int32),
            np.zeros(ne.value, np.int32), np.zeros(ne.value), np.zeros(lp.nrows, np.int32)]
    r = L.acdalm_sell_copy(m.h, 0, ctypes.byref(ns), ctypes.byref(short),
                           *[x.ctypes.data_as(ctypes.c_void_p) for x in bufs])
    assert r < 0
    m.free()
