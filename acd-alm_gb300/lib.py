"""ctypes binding of libacdalm.so, the C-ABI library (include/*.h).

Mirrors the reference's C interface (spmv.h, approx.h, alm.h): the same
function names, argument meaning and return values, with numpy arrays in
place of raw pointers.  Loading fails loudly if the library was not built;
nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("ACDALM_LIB", os.path.join(HERE, "libacdalm.so"))

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_sz = C.c_size_t
_vp = C.c_void_p

SPMV_SELL, SPMV_BLOCK, SPMV_CSR, SPMV_SELL_FMA = 0, 1, 2, 3
PRECISION_FP64, PRECISION_MIXED, PRECISION_AUTO = 0, 1, 2

ERRORS = {-1: "ACDALM_ECUDA", -2: "ACDALM_ETIMEOUT", -3: "ACDALM_ENOMEM",
          -4: "ACDALM_EINVAL", -5: "ACDALM_ENONFINITE", -6: "ACDALM_ENODEV",
          -7: "ACDALM_ETIMELIMIT"}


class Stats(C.Structure):
    _fields_ = [("seconds", C.c_double), ("inner_iterations", C.c_uint64),
                ("outer_iterations", C.c_uint64), ("rel_kkt", C.c_double),
                ("primal", C.c_double), ("dual", C.c_double), ("gap", C.c_double),
                ("objective", C.c_double), ("status", C.c_int),
                ("precision", C.c_int), ("fp32_inner_iterations", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AcdalmError(RuntimeError):
    pass


def load(path: str = LIB_PATH) -> C.CDLL:
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with acd-alm_gb300/build_lib.py "
            "(there is no CPU fallback)")
    L = C.CDLL(path)
    L.sparse_matrix_init.restype = None
    L.sparse_matrix_make.restype = _vp
    L.sparse_matrix_make.argtypes = [_sz, _sz, _sz, _u32p, _u32p, _f64p, C.c_int]
    L.sparse_matrix_copy.restype = _vp
    L.sparse_matrix_copy.argtypes = [_vp, C.c_int]
    L.sparse_matrix_free.argtypes = [_vp]
    for f in ("ncolumns", "nrows", "nnz"):
        getattr(L, "sparse_matrix_" + f).restype = _sz
        getattr(L, "sparse_matrix_" + f).argtypes = [_vp]
    for f in ("rows", "columns"):
        getattr(L, "sparse_matrix_" + f).restype = C.POINTER(C.c_uint32)
        getattr(L, "sparse_matrix_" + f).argtypes = [_vp]
    L.sparse_matrix_values.restype = C.POINTER(C.c_double)
    L.sparse_matrix_values.argtypes = [_vp]
    L.sparse_matrix_row_permute.argtypes = [_vp, _f64p, _sz, _f64p, C.c_int]
    L.sparse_matrix_col_permute.argtypes = [_vp, _f64p, _sz, _f64p, C.c_int]
    L.sparse_matrix_multiply.argtypes = [_f64p, _sz, _vp, _f64p, _sz, C.c_int, _vp]
    L.sparse_matrix_multiply_2.argtypes = [C.POINTER(C.POINTER(C.c_double)), _sz, _vp,
                                           C.POINTER(C.POINTER(C.c_double)), _sz,
                                           C.c_int, _vp]
    L.approx_make.restype = _vp
    L.approx_make.argtypes = [_vp, _sz, _f64p, _vp, _sz, _vp, _vp, _vp]
    L.approx_free.argtypes = [_vp]
    for f in ("rhs", "weight", "linear", "lower", "upper"):
        getattr(L, "approx_" + f).restype = C.POINTER(C.c_double)
        getattr(L, "approx_" + f).argtypes = [_vp]
    L.approx_update.argtypes = [_vp]
    for f in ("approx_solve", "mpg_solve", "cd_solve"):
        getattr(L, f).argtypes = [_f64p, _sz, _vp, _sz, C.c_double, C.c_double,
                                  C.c_double, _vp, _sz, _f64p, C.c_double, _vp]
    L.alm_make.restype = _vp
    L.alm_make.argtypes = [_vp, _sz, _f64p, _sz, _f64p, _vp, _vp, _vp, _vp]
    L.alm_free.argtypes = [_vp]
    L.alm_matrix.restype = _vp
    L.alm_matrix.argtypes = [_vp]
    for f in ("nrhs", "nvars"):
        getattr(L, "alm_" + f).restype = _sz
        getattr(L, "alm_" + f).argtypes = [_vp]
    L.acdalm_write_binary.argtypes = [_vp, _vp]
    L.acdalm_read_binary.restype = _vp
    L.acdalm_read_binary.argtypes = [_vp]
    L.acdalm_read_mps.restype = _vp
    L.acdalm_read_mps.argtypes = [_vp]
    L.alm_solve.argtypes = [_vp, _sz, _f64p, _sz, _f64p, _sz, _vp, _f64p, _vp]
    for f in ("rhs", "linear", "lower", "upper", "lambda_lower", "lambda_upper"):
        getattr(L, "alm_" + f).restype = C.POINTER(C.c_double)
        getattr(L, "alm_" + f).argtypes = [_vp]
    L.alm_set_precision.argtypes = [_vp, C.c_int]
    L.alm_set_kkt_tolerance.argtypes = [_vp, C.c_double]
    L.alm_set_inner_budget.argtypes = [_vp, C.c_uint64]
    L.alm_last_stats.argtypes = [_vp, C.POINTER(Stats)]
    L.alm_set_trace.argtypes = [_vp, C.c_uint64, C.c_uint64]
    L.acdalm_autotune.argtypes = [_vp, _sz, C.POINTER(C.c_int)]
    L.alm_trace_copy.argtypes = [_vp, _vp, _sz, C.POINTER(_sz), C.POINTER(_sz)]
    L.approx_last_stats.argtypes = [_vp, C.POINTER(Stats)]
    L.alm_stream.restype = _vp
    L.alm_stream.argtypes = [_vp]
    L.acdalm_last_error.restype = C.c_char_p
    L.acdalm_spmv_variant.argtypes = [C.c_int]
    L.acdalm_spmv_device.argtypes = [_vp, C.c_int, C.c_int, _vp, _vp, _vp]
    L.acdalm_spmv_device_f32.argtypes = [_vp, C.c_int, C.c_int, _vp, _vp, _vp]
    L.acdalm_matrix_device_bytes.restype = _sz
    L.acdalm_matrix_device_bytes.argtypes = [_vp]
    L.acdalm_block_bytes.restype = _sz
    L.acdalm_block_bytes.argtypes = [_vp, C.c_int, C.POINTER(_sz)]
    L.acdalm_block_copy.argtypes = [_vp, C.c_int, _u64p, _vp, _sz]
    L.acdalm_csr_copy.argtypes = [_vp, C.c_int, _u32p, _u32p, _f64p]
    L.acdalm_perm_copy.argtypes = [_vp, C.c_int, _u32p, _u32p]
    L.acdalm_sell_copy.argtypes = [_vp, C.c_int, C.POINTER(_sz), C.POINTER(_sz), _vp, _vp,
                                   _vp, _vp, _vp]
    L.acdalm_approx_permuted_matrix.restype = _vp
    L.acdalm_approx_permuted_matrix.argtypes = [_vp]
    L.acdalm_approx_step_sizes.argtypes = [_vp, _f64p, _f64p, _f64p]
    L.acdalm_batch_make.restype = _vp
    L.acdalm_batch_make.argtypes = [_vp, _sz]
    L.acdalm_batch_solve.argtypes = [_vp, _sz, _vp, _vp, _vp, _vp]
    L.acdalm_batch_seconds.restype = C.c_double
    L.acdalm_batch_seconds.argtypes = [_vp]
    L.acdalm_batch_free.argtypes = [_vp]
    L.acdalm_alm_approx.restype = _vp
    L.acdalm_alm_approx.argtypes = [_vp]
    L.acdalm_launch_count.restype = C.c_ulonglong
    L.acdalm_set_rounding.argtypes = [C.c_int]
    L.acdalm_server_create.restype = _vp
    L.acdalm_server_create.argtypes = [_sz, C.c_int, C.c_int, C.c_double, C.c_int]
    L.acdalm_server_submit.restype = C.c_longlong
    L.acdalm_server_submit.argtypes = [_vp, _sz, _sz, _sz, _u32p, _u32p, _f64p, _f64p, _vp,
                                       _vp, _vp, _vp, _vp]
    L.acdalm_server_poll.argtypes = [_vp, _vp, C.c_int, C.c_double]
    L.acdalm_server_result.argtypes = [_vp, C.c_longlong, _vp, _vp, C.POINTER(Stats),
                                       C.POINTER(C.c_double)]
    L.acdalm_server_destroy.argtypes = [_vp]
    L.acdalm_server_set_inner_budget.argtypes = [_vp, C.c_uint64]
    L.thread_pool_init.restype = _vp
    L.thread_pool_init.argtypes = [C.c_uint]
    L.thread_pool_free.argtypes = [_vp]
    L.thread_pool_count.restype = _sz
    L.thread_pool_count.argtypes = [_vp]
    return L


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
        _lib.sparse_matrix_init()
    return _lib


def check(ret: int, what: str) -> int:
    if ret < 0:
        msg = lib().acdalm_last_error().decode()
        raise AcdalmError(f"{what}: {ERRORS.get(ret, ret)}: {msg}")
    return ret


def _ptr(a):
    return None if a is None else np.ascontiguousarray(a, np.float64).ctypes.data_as(_vp)


class Matrix:
    """sparse_matrix_t (spmv.h)."""

    def __init__(self, lp=None, permute: bool = False, handle=None, owner=True):
        L = lib()
        if handle is not None:
            self.h, self.owner = handle, owner
        else:
            self.h = L.sparse_matrix_make(lp.ncols, lp.nrows, lp.nnz,
                                          np.ascontiguousarray(lp.rows, np.uint32),
                                          np.ascontiguousarray(lp.cols, np.uint32),
                                          np.ascontiguousarray(lp.vals, np.float64),
                                          int(permute))
            self.owner = True
            if not self.h:
                raise AcdalmError(lib().acdalm_last_error().decode())
        self.nrows = L.sparse_matrix_nrows(self.h)
        self.ncols = L.sparse_matrix_ncolumns(self.h)
        self.nnz = L.sparse_matrix_nnz(self.h)

    def free(self):
        if self.h and self.owner:
            lib().sparse_matrix_free(self.h)
        self.h = None

    def coo(self):
        L = lib()
        n = self.nnz
        r = np.ctypeslib.as_array(L.sparse_matrix_rows(self.h), (max(n, 1),))[:n].copy()
        c = np.ctypeslib.as_array(L.sparse_matrix_columns(self.h), (max(n, 1),))[:n].copy()
        v = np.ctypeslib.as_array(L.sparse_matrix_values(self.h), (max(n, 1),))[:n].copy()
        return r, c, v

    def layouts(self) -> dict:
        """CSR, block arenas, permutations and the Z-order COO (the same
        keys as the oracle's Lib.layouts)."""
        L = lib()
        out = {"coo": self.coo()}
        for t, n in ((0, self.nrows), (1, self.ncols)):
            ri = np.zeros(n + 1, np.uint32)
            cc = np.zeros(self.nnz, np.uint32)
            vv = np.zeros(self.nnz)
            L.acdalm_csr_copy(self.h, t, ri, cc, vv)
            out[f"csr{t}"] = (ri, cc, vv)
            nb = _sz()
            nbytes = L.acdalm_block_bytes(self.h, t, C.byref(nb))
            offs = np.zeros(max(nb.value, 1), np.uint64)
            arena = np.zeros(max(nbytes, 1), np.uint8)
            L.acdalm_block_copy(self.h, t, offs, arena.ctypes.data_as(_vp), nbytes)
            out[f"block{t}"] = (offs[:nb.value], arena[:nbytes])
        for row, n in ((1, self.nrows), (0, self.ncols)):
            idx = np.zeros(n, np.uint32)
            ridx = np.zeros(n, np.uint32)
            L.acdalm_perm_copy(self.h, row, idx, ridx)
            out["rperm" if row else "cperm"] = (idx, ridx)
        return out

    def sell(self, transpose: bool) -> dict:
        """The SELL layout of A (or A') the SELL SpMV variant uploads:
        ptr, row0, col, val and row_of_d (device row -> matrix row)."""
        L = lib()
        ns, ne = _sz(), _sz()
        check(L.acdalm_sell_copy(self.h, int(transpose), C.byref(ns), C.byref(ne),
                                 None, None, None, None, None), "acdalm_sell_copy")
        nrows = self.ncols if transpose else self.nrows
        out = {"ptr": np.zeros(ns.value + 1, np.int64),
               "row0": np.zeros(max(ns.value, 1), np.int32),
               "col": np.zeros(max(ne.value, 1), np.int32),
               "val": np.zeros(max(ne.value, 1)),
               "row_of_d": np.zeros(max(nrows, 1), np.int32)}
        check(L.acdalm_sell_copy(self.h, int(transpose), C.byref(ns), C.byref(ne),
                                 *(out[k].ctypes.data_as(_vp)
                                   for k in ("ptr", "row0", "col", "val", "row_of_d"))),
              "acdalm_sell_copy")
        out["row0"] = out["row0"][:ns.value]
        out["col"] = out["col"][:ne.value]
        out["val"] = out["val"][:ne.value]
        out["row_of_d"] = out["row_of_d"][:nrows]
        return out

    def multiply(self, x, transpose=False):
        ny = self.ncols if transpose else self.nrows
        y = np.zeros(ny)
        x = np.ascontiguousarray(x, np.float64)
        check(lib().sparse_matrix_multiply(y, ny, self.h, x, x.shape[0], int(transpose),
                                           None), "sparse_matrix_multiply")
        return y

    def multiply_2(self, x0, x1, transpose=False):
        ny = self.ncols if transpose else self.nrows
        ys = [np.zeros(ny), np.zeros(ny)]
        xs = [np.ascontiguousarray(x0, np.float64), np.ascontiguousarray(x1, np.float64)]
        DP = C.POINTER(C.c_double)
        ya = (DP * 2)(*[y.ctypes.data_as(DP) for y in ys])
        xa = (DP * 2)(*[x.ctypes.data_as(DP) for x in xs])
        check(lib().sparse_matrix_multiply_2(ya, ny, self.h, xa, xs[0].shape[0],
                                             int(transpose), None),
              "sparse_matrix_multiply_2")
        return ys


class Approx:
    """approx_t (approx.h)."""

    def __init__(self, matrix: Matrix, lp, weight=None, linear=True):
        L = lib()
        self._keep = [np.ascontiguousarray(a, np.float64) for a in
                      (lp.rhs, weight if weight is not None else np.ones(lp.nrows),
                       lp.linear, lp.lower, lp.upper)]
        self.h = L.approx_make(matrix.h, lp.nrows, self._keep[0],
                               _ptr(self._keep[1]) if weight is not None else None,
                               lp.ncols, _ptr(self._keep[2]) if linear else None,
                               _ptr(self._keep[3]), _ptr(self._keep[4]))
        if not self.h:
            raise AcdalmError(lib().acdalm_last_error().decode())
        self.nrows, self.ncols = lp.nrows, lp.ncols

    def free(self):
        if self.h:
            lib().approx_free(self.h)
        self.h = None

    def vec(self, name):
        n = self.nrows if name in ("rhs", "weight") else self.ncols
        p = getattr(lib(), "approx_" + name)(self.h)
        return np.ctypeslib.as_array(p, (max(n, 1),))[:n]

    def update(self):
        return lib().approx_update(self.h)

    def permuted_matrix(self) -> Matrix:
        return Matrix(handle=lib().acdalm_approx_permuted_matrix(self.h), owner=False)

    def step_sizes(self):
        beta = np.zeros(self.nrows)
        v = np.zeros(self.ncols)
        inv_v = np.zeros(self.ncols)
        check(lib().acdalm_approx_step_sizes(self.h, beta, v, inv_v), "step sizes")
        return beta, v, inv_v

    def _solve(self, fn, x, niter, max_pg, max_value, min_delta, log, period, offset):
        diag = np.zeros(5)
        x = np.ascontiguousarray(x, np.float64).copy()
        f = _open_log(log)
        try:
            r = check(getattr(lib(), fn)(x, self.ncols, self.h, niter, max_pg, max_value,
                                         min_delta, f, period, diag, offset, None), fn)
        finally:
            _close_log(f)
        return r, x, diag

    def solve(self, x, niter, max_pg=0.0, max_value=-np.inf, min_delta=0.0, log=None,
              period=0, offset=0.0):
        return self._solve("approx_solve", x, niter, max_pg, max_value, min_delta, log,
                           period, offset)

    def mpg_solve(self, x, niter, max_pg=0.0, max_value=-np.inf, log=None, period=0,
                  offset=0.0):
        return self._solve("mpg_solve", x, niter, max_pg, max_value, 0.0, log, period,
                           offset)

    def stats(self) -> dict:
        s = Stats()
        lib().approx_last_stats(self.h, C.byref(s))
        return s.as_dict()


class Alm:
    """alm_t (alm.h)."""

    def __init__(self, matrix: Matrix, lp):
        L = lib()
        self._keep = [np.ascontiguousarray(a, np.float64) for a in
                      (lp.lower, lp.upper, lp.lambda_lower, lp.lambda_upper)]
        self.h = L.alm_make(matrix.h, lp.nrows, np.ascontiguousarray(lp.rhs, np.float64),
                            lp.ncols, np.ascontiguousarray(lp.linear, np.float64),
                            *[_ptr(k) for k in self._keep])
        if not self.h:
            raise AcdalmError(lib().acdalm_last_error().decode())
        self.nrows, self.ncols = lp.nrows, lp.ncols

    def free(self):
        if self.h:
            lib().alm_free(self.h)
        self.h = None

    def set_precision(self, mode: int):
        check(lib().alm_set_precision(self.h, mode), "alm_set_precision")

    def set_kkt_tolerance(self, tol: float):
        check(lib().alm_set_kkt_tolerance(self.h, tol), "alm_set_kkt_tolerance")

    def set_inner_budget(self, budget: int):
        check(lib().alm_set_inner_budget(self.h, int(budget)), "alm_set_inner_budget")

    def solve(self, niter=1000, x=None, lam=None, log=None):
        x = np.zeros(self.ncols) if x is None else np.ascontiguousarray(x, np.float64).copy()
        lam = (np.zeros(self.nrows) if lam is None
               else np.ascontiguousarray(lam, np.float64).copy())
        diag = np.zeros(3)
        f = _open_log(log)
        try:
            r = check(lib().alm_solve(self.h, niter, x, self.ncols, lam, self.nrows, f, diag,
                                      None), "alm_solve")
        finally:
            _close_log(f)
        return r, x, lam, diag

    def stats(self) -> dict:
        s = Stats()
        lib().alm_last_stats(self.h, C.byref(s))
        return s.as_dict()

    def autotune(self, iterations: int = 300) -> int:
        """acdalm_autotune: the step cap chosen for this instance's layout."""
        chosen = C.c_int(-1)
        check(lib().acdalm_autotune(self.h, iterations, C.byref(chosen)), "acdalm_autotune")
        return chosen.value

    def set_trace(self, first: int, count: int):
        check(lib().alm_set_trace(self.h, first, count), "alm_set_trace")

    def trace(self) -> np.ndarray:
        """Phase stamps of the last traced solve: [reduction, cta, phase] ns."""
        ctas, count = _sz(), _sz()
        check(lib().alm_trace_copy(self.h, None, 0, C.byref(ctas), C.byref(count)),
              "alm_trace_copy")
        out = np.zeros(ctas.value * count.value * 3, np.uint64)
        if out.size:
            check(lib().alm_trace_copy(self.h, out.ctypes.data_as(_vp), out.size,
                                       C.byref(ctas), C.byref(count)), "alm_trace_copy")
        return out.reshape(count.value, ctas.value, 3)

    def stream(self) -> int:
        return lib().alm_stream(self.h) or 0


_libc = None


def _open_log(path):
    global _libc
    if path is None:
        return None
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.fopen.restype = _vp
        _libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        _libc.fclose.argtypes = [_vp]
    return _libc.fopen(path.encode(), b"w")


def _close_log(f):
    if f:
        _libc.fclose(f)


class Batch:
    """acdalm_batch_t: alm_solve on many Alm instances in one launch."""

    def __init__(self, alms):
        self.alms = list(alms)
        arr = (_vp * max(len(self.alms), 1))(*[a.h for a in self.alms])
        self.h = lib().acdalm_batch_make(arr, len(self.alms))
        if not self.h:
            raise AcdalmError(lib().acdalm_last_error().decode())

    def solve(self, niter=1000, xs=None, lams=None):
        n = len(self.alms)
        xs = [np.zeros(a.ncols) if xs is None else np.ascontiguousarray(xs[i], np.float64).copy()
              for i, a in enumerate(self.alms)]
        lams = [np.zeros(a.nrows) if lams is None else np.ascontiguousarray(lams[i], np.float64).copy()
                for i, a in enumerate(self.alms)]
        DP = C.POINTER(C.c_double)
        xa = (DP * max(n, 1))(*[x.ctypes.data_as(DP) for x in xs])
        la = (DP * max(n, 1))(*[l.ctypes.data_as(DP) for l in lams])
        ret = np.zeros(max(n, 1), np.int32)
        diag = np.zeros(3 * max(n, 1))
        r = lib().acdalm_batch_solve(self.h, niter, C.cast(xa, _vp), C.cast(la, _vp),
                                     ret.ctypes.data_as(_vp), diag.ctypes.data_as(_vp))
        check(r, "acdalm_batch_solve")
        return ret[:n], xs, lams, diag[:3 * n].reshape(n, 3)

    def seconds(self) -> float:
        return lib().acdalm_batch_seconds(self.h)

    def free(self):
        if self.h:
            lib().acdalm_batch_free(self.h)
        self.h = None


class Server:
    """acdalm_server_t: continuous batching of LP solves."""

    def __init__(self, device_budget=0, max_inflight=0, precision=PRECISION_MIXED,
                 kkt_tol=1e-6, builder_threads=0):
        self.h = lib().acdalm_server_create(device_budget, max_inflight, precision, kkt_tol,
                                            builder_threads)
        if not self.h:
            raise AcdalmError(lib().acdalm_last_error().decode())
        self.shapes = {}

    def submit(self, lp) -> int:
        keep = [np.ascontiguousarray(a, np.float64) for a in
                (lp.linear, lp.lower, lp.upper, lp.lambda_lower, lp.lambda_upper)]
        rid = lib().acdalm_server_submit(
            self.h, lp.nrows, lp.ncols, lp.nnz, np.ascontiguousarray(lp.rows, np.uint32),
            np.ascontiguousarray(lp.cols, np.uint32), np.ascontiguousarray(lp.vals, np.float64),
            np.ascontiguousarray(lp.rhs, np.float64), *[_ptr(k) for k in keep])
        check(rid, "acdalm_server_submit")
        self.shapes[rid] = (lp.nrows, lp.ncols)
        return rid

    def poll(self, timeout=0.0, cap=1024):
        ids = np.zeros(cap, np.int64)
        n = lib().acdalm_server_poll(self.h, ids.ctypes.data_as(_vp), cap, timeout)
        return [int(i) for i in ids[:n]]

    def result(self, rid):
        m, n = self.shapes.pop(rid)
        x = np.zeros(n)
        lam = np.zeros(m)
        st = Stats()
        lat = C.c_double()
        r = lib().acdalm_server_result(self.h, rid, x.ctypes.data_as(_vp),
                                       lam.ctypes.data_as(_vp), C.byref(st), C.byref(lat))
        return r, x, lam, st.as_dict(), lat.value

    def set_inner_budget(self, budget: int):
        check(lib().acdalm_server_set_inner_budget(self.h, budget),
              "acdalm_server_set_inner_budget")

    def close(self):
        if self.h:
            lib().acdalm_server_destroy(self.h)
        self.h = None
