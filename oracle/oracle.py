"""ctypes bindings for the oracle (test infrastructure only).

Two libraries share one Python interface:

* ``Lib("oracle")`` -- my C restatement of the reference (``_build/liboracle.so``),
  available everywhere (built by ``make oracle``).
* ``Lib("ref")`` -- the reference compiled from its own sources plus
  ``ref_shim.c`` (``_ref/libacdref.so``), available only where the reference
  sources were present at build time.

Only tests/, ``__graft_entry__.smoke()`` and the CPU baseline of bench.py
import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {"oracle": os.path.join(HERE, "_build", "liboracle.so"),
         "ref": os.path.join(HERE, "_ref", "libacdref.so")}

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_sz = C.c_size_t
_vp = C.c_void_p


def build(ref: bool = True) -> None:
    """Compile the oracle (and the reference when its sources exist)."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def available(kind: str) -> bool:
    return os.path.exists(PATHS[kind])


class Lib:
    """Uniform view over the oracle restatement and the compiled reference."""

    def __init__(self, kind: str = "oracle"):
        self.kind = kind
        self.lib = C.CDLL(PATHS[kind])
        L = self.lib
        p = "or_" if kind == "oracle" else ""
        self.p = p
        if kind == "oracle":
            L.or_matrix_make.restype = _vp
            L.or_matrix_make.argtypes = [_sz, _sz, _sz, _u32p, _u32p, _f64p, C.c_int]
            L.or_matrix_free.argtypes = [_vp]
            L.or_approx_make.restype = _vp
            L.or_approx_make.argtypes = [_vp, _sz, _f64p, _vp, _sz, _vp, _vp, _vp]
            L.or_approx_free.argtypes = [_vp]
            L.or_approx_update.argtypes = [_vp]
            L.or_approx_vec.restype = C.POINTER(C.c_double)
            L.or_approx_vec.argtypes = [_vp, C.c_int]
            L.or_alm_make.restype = _vp
            L.or_alm_make.argtypes = [_vp, _sz, _f64p, _sz, _f64p, _vp, _vp, _vp, _vp]
            L.or_alm_free.argtypes = [_vp]
            L.or_alm_approx.restype = _vp
            L.or_alm_approx.argtypes = [_vp]
            L.or_alm_solve.argtypes = [_vp, _sz, _f64p, _f64p, C.c_char_p, _f64p,
                                       _sz, C.POINTER(_sz)]
            L.or_approx_solve.argtypes = [_vp, _f64p, _sz, C.c_double, C.c_double,
                                          C.c_double, C.c_char_p, _sz, _f64p,
                                          C.c_double, _vp, _sz]
            L.or_mpg_solve.argtypes = [_vp, _f64p, _sz, C.c_double, C.c_double,
                                       C.c_double, C.c_char_p, _sz, _f64p,
                                       C.c_double]
            L.or_set_threads.argtypes = [C.c_int]
            L.or_multiply.argtypes = [_f64p, _vp, _f64p, C.c_int]
            L.or_multiply_csr.argtypes = [_f64p, _vp, _f64p, C.c_int]
            L.or_k_violation.restype = C.c_double
            L.or_k_violation.argtypes = [_vp, C.c_int, _f64p, _f64p]
            L.or_k_gradient.argtypes = [_vp, C.c_int, _f64p, _f64p]
            L.or_k_gradient2_step.restype = C.c_double
            L.or_k_gradient2_step.argtypes = [_vp, C.c_int, _f64p, _f64p, _f64p,
                                              C.c_double, _f64p, _f64p, _f64p]
            L.or_k_gradient_long_step.restype = C.c_double
            L.or_k_gradient_long_step.argtypes = [_vp, C.c_int, C.c_int, _f64p,
                                                  _f64p, _f64p, C.c_double,
                                                  C.c_double, _vp, _f64p, _f64p]
            L.or_k_linterp_xy.argtypes = [_sz, _sz, _f64p, _f64p, _f64p, _f64p,
                                          _f64p, C.c_double, C.c_double]
            L.or_k_project_gradient_norm.restype = C.c_double
            L.or_k_project_gradient_norm.argtypes = [_vp, C.c_int, _f64p, _f64p]
            L.or_k_dot_diff.restype = C.c_double
            L.or_k_dot_diff.argtypes = [_sz, _f64p, _f64p, _f64p]
        else:
            L.sparse_matrix_init()
            L.sparse_matrix_make.restype = _vp
            L.sparse_matrix_make.argtypes = [_sz, _sz, _sz, _u32p, _u32p, _f64p, C.c_int]
            L.sparse_matrix_free.argtypes = [_vp]
            L.sparse_matrix_multiply.argtypes = [_f64p, _sz, _vp, _f64p, _sz,
                                                 C.c_int, _vp]
            L.approx_make.restype = _vp
            L.approx_make.argtypes = [_vp, _sz, _f64p, _vp, _sz, _vp, _vp, _vp]
            L.approx_free.argtypes = [_vp]
            L.approx_update.argtypes = [_vp]
            for acc in ("rhs", "weight", "linear", "lower", "upper"):
                f = getattr(L, "approx_" + acc)
                f.restype = C.POINTER(C.c_double)
                f.argtypes = [_vp]
            L.ref_approx_permuted_matrix.restype = _vp
            L.ref_approx_permuted_matrix.argtypes = [_vp]
            L.alm_make.restype = _vp
            L.alm_make.argtypes = [_vp, _sz, _f64p, _sz, _f64p, _vp, _vp, _vp, _vp]
            L.alm_free.argtypes = [_vp]
            L.ref_alm_solve.argtypes = [_vp, _sz, _f64p, _f64p, C.c_char_p, _f64p,
                                        C.c_int]
            L.ref_approx_solve.argtypes = [_vp, _f64p, _sz, C.c_double, C.c_double,
                                           C.c_double, C.c_char_p, _sz, _f64p,
                                           C.c_double, C.c_int]
            L.ref_mpg_solve.argtypes = [_vp, _f64p, _sz, C.c_double, C.c_double,
                                        C.c_double, C.c_char_p, _sz, _f64p,
                                        C.c_double, C.c_int]
            L.ref_set_inner_budget.argtypes = [_sz]
            L.ref_alm_solve_kkt.argtypes = [_vp, _sz, _f64p, _f64p, C.c_double, _f64p,
                                            C.POINTER(_sz), C.c_int]
            L.ref_inner_used.restype = _sz
            L.ref_approx_internals.argtypes = [_vp, C.c_int, _u32p, _f64p, _f64p,
                                               _f64p, _f64p, _f64p, _f64p, _f64p]
        pre = "or_" if kind == "oracle" else "ref_"
        getattr(L, pre + "matrix_dims").argtypes = [_vp, C.POINTER(_sz),
                                                    C.POINTER(_sz), C.POINTER(_sz)]
        getattr(L, pre + "coo").argtypes = [_vp, _u32p, _u32p, _f64p]
        getattr(L, pre + "csr").argtypes = [_vp, C.c_int, _u32p, _u32p, _f64p]
        getattr(L, pre + "block_bytes").restype = _sz
        getattr(L, pre + "block_bytes").argtypes = [_vp, C.c_int, C.POINTER(_sz)]
        getattr(L, pre + "block").argtypes = [_vp, C.c_int, _u64p, _vp, _sz]
        getattr(L, pre + "perm").argtypes = [_vp, C.c_int, _u32p, _u32p]
        self.pre = pre

    # ---- matrices ----
    def matrix(self, lp, permute: bool = False):
        f = self.lib.or_matrix_make if self.kind == "oracle" else self.lib.sparse_matrix_make
        return f(lp.ncols, lp.nrows, lp.nnz, np.ascontiguousarray(lp.rows, np.uint32),
                 np.ascontiguousarray(lp.cols, np.uint32),
                 np.ascontiguousarray(lp.vals, np.float64), int(permute))

    def matrix_free(self, m):
        (self.lib.or_matrix_free if self.kind == "oracle" else self.lib.sparse_matrix_free)(m)

    def dims(self, m):
        a, b, c = _sz(), _sz(), _sz()
        getattr(self.lib, self.pre + "matrix_dims")(m, a, b, c)
        return a.value, b.value, c.value

    def layouts(self, m) -> dict:
        """Every internal layout of a matrix, as numpy arrays."""
        nrows, ncols, nnz = self.dims(m)
        L, pre = self.lib, self.pre
        out = {}
        r = np.zeros(nnz, np.uint32); c = np.zeros(nnz, np.uint32); v = np.zeros(nnz)
        getattr(L, pre + "coo")(m, r, c, v)
        out["coo"] = (r, c, v)
        for t, n in ((0, nrows), (1, ncols)):
            ri = np.zeros(n + 1, np.uint32); cc = np.zeros(nnz, np.uint32); vv = np.zeros(nnz)
            getattr(L, pre + "csr")(m, t, ri, cc, vv)
            out[f"csr{t}"] = (ri, cc, vv)
            nb = _sz()
            nbytes = getattr(L, pre + "block_bytes")(m, t, nb)
            offs = np.zeros(max(nb.value, 1), np.uint64)
            arena = np.zeros(max(nbytes, 1), np.uint8)
            getattr(L, pre + "block")(m, t, offs, arena.ctypes.data_as(_vp), nbytes)
            out[f"block{t}"] = (offs[:nb.value], arena[:nbytes])
        for row, n in ((1, nrows), (0, ncols)):
            idx = np.zeros(n, np.uint32); ridx = np.zeros(n, np.uint32)
            getattr(L, pre + "perm")(m, row, idx, ridx)
            out["rperm" if row else "cperm"] = (idx, ridx)
        return out

    def multiply(self, m, x, transpose: bool):
        nrows, ncols, _ = self.dims(m)
        ny = ncols if transpose else nrows
        y = np.zeros(ny)
        x = np.ascontiguousarray(x, np.float64)
        if self.kind == "oracle":
            self.lib.or_multiply(y, m, x, int(transpose))
        else:
            self.lib.sparse_matrix_multiply(y, ny, m, x, x.shape[0], int(transpose), None)
        return y

    # ---- approx ----
    def approx(self, m, lp, weight=None, linear=True):
        f = self.lib.or_approx_make if self.kind == "oracle" else self.lib.approx_make
        keep = [np.ascontiguousarray(a, np.float64) for a in
                (weight if weight is not None else np.ones(lp.nrows),
                 lp.linear, lp.lower, lp.upper)]
        w = keep[0].ctypes.data_as(_vp) if weight is not None else None
        a = f(m, lp.nrows, np.ascontiguousarray(lp.rhs, np.float64), w, lp.ncols,
              keep[1].ctypes.data_as(_vp) if linear else None,
              keep[2].ctypes.data_as(_vp), keep[3].ctypes.data_as(_vp))
        return a

    def approx_free(self, a):
        (self.lib.or_approx_free if self.kind == "oracle" else self.lib.approx_free)(a)

    def internals(self, a, nrows, ncols, permuted: bool):
        beta = np.zeros(nrows, np.uint32)
        arrs = [np.zeros(ncols), np.zeros(ncols), np.zeros(nrows), np.zeros(nrows),
                np.zeros(ncols), np.zeros(ncols), np.zeros(ncols)]
        f = (self.lib.or_approx_internals if self.kind == "oracle"
             else self.lib.ref_approx_internals)
        if self.kind == "oracle":
            self.lib.or_approx_internals.argtypes = [_vp, C.c_int, _u32p] + [_f64p] * 7
        f(a, int(permuted), beta, *arrs)
        names = ["v", "inv_v", "rhs", "weight", "linear", "lower", "upper"]
        d = dict(zip(names, arrs))
        d["beta"] = beta
        return d

    def approx_solve(self, a, x, niter, max_pg=0.0, max_value=-np.inf,
                     min_delta=0.0, log=None, period=0, offset=0.0, threads=1):
        diag = np.zeros(5)
        x = np.ascontiguousarray(x, np.float64).copy()
        logb = log.encode() if log else None
        if self.kind == "oracle":
            self.lib.or_set_threads(threads)
            r = self.lib.or_approx_solve(a, x, niter, max_pg, max_value, min_delta,
                                         logb, period, diag, offset, None, 0)
        else:
            r = self.lib.ref_approx_solve(a, x, niter, max_pg, max_value, min_delta,
                                          logb, period, diag, offset,
                                          threads if threads > 1 else 0)
        return r, x, diag

    def mpg_solve(self, a, x, niter, max_pg=0.0, max_value=-np.inf, log=None,
                  period=0, offset=0.0):
        diag = np.zeros(5)
        x = np.ascontiguousarray(x, np.float64).copy()
        logb = log.encode() if log else None
        if self.kind == "oracle":
            r = self.lib.or_mpg_solve(a, x, niter, max_pg, max_value, 0.0, logb,
                                      period, diag, offset)
        else:
            r = self.lib.ref_mpg_solve(a, x, niter, max_pg, max_value, 0.0, logb,
                                       period, diag, offset, 0)
        return r, x, diag

    # ---- alm ----
    def alm(self, m, lp):
        f = self.lib.or_alm_make if self.kind == "oracle" else self.lib.alm_make
        keep = [np.ascontiguousarray(a, np.float64) for a in
                (lp.lower, lp.upper, lp.lambda_lower, lp.lambda_upper)]
        h = f(m, lp.nrows, np.ascontiguousarray(lp.rhs, np.float64), lp.ncols,
              np.ascontiguousarray(lp.linear, np.float64),
              *[k.ctypes.data_as(_vp) for k in keep])
        return h

    def alm_free(self, h):
        (self.lib.or_alm_free if self.kind == "oracle" else self.lib.alm_free)(h)

    def alm_solve(self, h, nrows, ncols, niter=1000, x=None, lam=None, log=None,
                  inner_budget=None, threads=1):
        x = np.zeros(ncols) if x is None else np.ascontiguousarray(x, np.float64).copy()
        lam = np.zeros(nrows) if lam is None else np.ascontiguousarray(lam, np.float64).copy()
        diag = np.zeros(3)
        logb = log.encode() if log else None
        budget = (1 << 64) - 1 if inner_budget is None else int(inner_budget)
        if self.kind == "oracle":
            self.lib.or_set_threads(threads)
            used = _sz()
            r = self.lib.or_alm_solve(h, niter, x, lam, logb, diag, budget, used)
            used = used.value
        else:
            self.lib.ref_set_inner_budget(budget)
            r = self.lib.ref_alm_solve(h, niter, x, lam, logb, diag,
                                       threads if threads > 1 else 0)
            used = self.lib.ref_inner_used()
            self.lib.ref_set_inner_budget((1 << 64) - 1)
        return r, x, lam, diag, used

    def alm_solve_kkt(self, h, nrows, ncols, tol, niter=1000, threads=1):
        """The reference's alm_solve stopped at relative KKT <= tol (checked
        at the start of every outer iteration after the first); reference
        library only.  Returns (ret, x, lambda, [primal, dual, gap, c'x],
        outer iterations, inner iterations)."""
        assert self.kind == "ref"
        x = np.zeros(ncols)
        lam = np.zeros(nrows)
        kk = np.zeros(4)
        outer = _sz()
        self.lib.ref_set_inner_budget((1 << 64) - 1)
        r = self.lib.ref_alm_solve_kkt(h, niter, x, lam, tol, kk, C.byref(outer),
                                       threads if threads > 1 else 0)
        inner = self.lib.ref_inner_used()
        return r, x, lam, kk, outer.value, inner
