"""Seeded synthetic LP instances for the five workloads of this solver.

Every instance is ``min c'x  s.t.  A x = b,  l <= x <= u`` with optional
bounds on the multipliers, returned as a :class:`LP` holding a COO matrix
(``rows``/``cols`` uint32, ``vals`` float64) and float64 vectors, exactly what
``sparse_matrix_make`` + ``alm_make`` take (spmv/spmv.h:19-24, alm.h:43-47 of
the reference).  No public dataset is involved: all workloads are drawn from
numpy's PCG64 with a recorded seed.

Workloads (names used throughout the repository):

``small``     m=1,000, n=2,000, 5 distinct uniform rows per column, values
              U[-1,1], x0~U[0,10], b=A x0, c~U[-1,1], 0<=x<=10.
``mid``       m=100,000, n=200,000, column counts ~ Zipf(s=1.5) truncated to
              [1,200] then raised to >=2 (mean ~11.3, ~2.25M nnz), otherwise as
              ``small``.
``covering``  A x >= 1 with m=1,000,000, n=4,000,000, 8 ones per column in
              distinct uniform rows, an empty row gets one forced entry, c =
              uniform integers [1,100], 0<=x<=1; slacks make it [A -I][x;s]=1
              with s>=0 and multipliers >= 0.
``batch``     512 instances, m = floor(exp(U[ln 200, ln 20000])), n=2m, 6
              nonzeros per column, otherwise as ``small``.
``stream``    20,000 instances as ``batch`` with m in [500, 200,000] and
              Poisson arrival times at 2,000/s.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class LP:
    """One LP in the reference's input form (COO + dense vectors)."""

    nrows: int
    ncols: int
    rows: np.ndarray  # uint32[nnz]
    cols: np.ndarray  # uint32[nnz]
    vals: np.ndarray  # float64[nnz]
    rhs: np.ndarray  # float64[nrows]
    linear: np.ndarray  # float64[ncols]
    lower: np.ndarray  # float64[ncols]
    upper: np.ndarray  # float64[ncols]
    lambda_lower: np.ndarray  # float64[nrows]
    lambda_upper: np.ndarray  # float64[nrows]
    name: str = ""
    seed: int = 0

    @property
    def nnz(self) -> int:
        return int(self.vals.shape[0])

    def matvec(self, x: np.ndarray) -> np.ndarray:
        """A x in float64 (sequential per-row accumulation in COO order)."""
        return np.bincount(self.rows, weights=self.vals * x[self.cols],
                           minlength=self.nrows)

    def rmatvec(self, y: np.ndarray) -> np.ndarray:
        """A' y in float64."""
        return np.bincount(self.cols, weights=self.vals * y[self.rows],
                           minlength=self.ncols)

    def sha256(self) -> str:
        """SHA-256 over the arrays that define the LP, in a fixed order: a
        fixture made from a seeded instance stores it, so a test can tell
        that it rebuilt the same LP from the seed."""
        import hashlib
        h = hashlib.sha256()
        for a in (self.rows, self.cols, self.vals, self.rhs, self.linear, self.lower,
                  self.upper, self.lambda_lower, self.lambda_upper):
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()


def _distinct_rows(rng: np.random.Generator, m: int, counts: np.ndarray):
    """For column j draw counts[j] distinct rows uniformly from [0, m).

    Returns (rows, cols) with the entries of each column contiguous and rows
    ascending within a column."""
    counts = np.asarray(counts, dtype=np.int64)
    if counts.max(initial=0) > m:
        raise ValueError("more nonzeros per column than rows")
    rows_out = []
    cols_out = []
    for k in np.unique(counts):
        k = int(k)
        if k == 0:
            continue
        colset = np.nonzero(counts == k)[0]
        draw = rng.integers(0, m, size=(colset.size, k), dtype=np.int64)
        draw.sort(axis=1)
        while True:
            dup = np.zeros(draw.shape, dtype=bool)
            dup[:, 1:] = draw[:, 1:] == draw[:, :-1]
            bad = np.nonzero(dup.any(axis=1))[0]
            if bad.size == 0:
                break
            redo = rng.integers(0, m, size=int(dup[bad].sum()), dtype=np.int64)
            sub = draw[bad]
            sub[dup[bad]] = redo
            sub.sort(axis=1)
            draw[bad] = sub
        rows_out.append(draw.reshape(-1))
        cols_out.append(np.repeat(colset, k))
    rows = np.concatenate(rows_out) if rows_out else np.zeros(0, np.int64)
    cols = np.concatenate(cols_out) if cols_out else np.zeros(0, np.int64)
    order = np.lexsort((rows, cols))
    return rows[order].astype(np.uint32), cols[order].astype(np.uint32)


def _zipf_counts(rng: np.random.Generator, n: int, s: float = 1.5,
                 kmax: int = 200, kmin_raise: int = 2) -> np.ndarray:
    """Zipf(s) truncated to [1, kmax] by inverse CDF, then raised to >= 2."""
    k = np.arange(1, kmax + 1, dtype=np.float64)
    pmf = k ** (-s)
    cdf = np.cumsum(pmf / pmf.sum())
    u = rng.random(n)
    counts = np.searchsorted(cdf, u, side="right") + 1
    counts = np.minimum(counts, kmax)
    return np.maximum(counts, kmin_raise).astype(np.int64)


def _feasible_equality_lp(rng, m: int, n: int, counts, name: str, seed: int,
                          box_hi: float = 10.0) -> LP:
    rows, cols = _distinct_rows(rng, m, counts)
    vals = rng.uniform(-1.0, 1.0, size=rows.shape[0])
    x0 = rng.uniform(0.0, box_hi, size=n)
    c = rng.uniform(-1.0, 1.0, size=n)
    lp = LP(nrows=m, ncols=n, rows=rows, cols=cols, vals=vals,
            rhs=np.zeros(m), linear=c, lower=np.zeros(n),
            upper=np.full(n, box_hi), lambda_lower=np.full(m, -np.inf),
            lambda_upper=np.full(m, np.inf), name=name, seed=seed)
    lp.rhs = lp.matvec(x0)
    return lp


def small(seed: int = 1, m: int = 1000, n: int | None = None,
          per_col: int = 5) -> LP:
    """The small CPU-runnable LP: m=1,000, n=2,000, 5 nonzeros per column."""
    n = 2 * m if n is None else n
    rng = np.random.Generator(np.random.PCG64(seed))
    return _feasible_equality_lp(rng, m, n, np.full(n, per_col), "small", seed)


def mid(seed: int = 2, m: int = 100_000, n: int | None = None) -> LP:
    """The mid-size LP: m=100,000, n=200,000, Zipf(1.5) column counts."""
    n = 2 * m if n is None else n
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.minimum(_zipf_counts(rng, n), m)
    return _feasible_equality_lp(rng, m, n, counts, "mid", seed)


def covering(seed: int = 3, m: int = 1_000_000, n: int = 4_000_000,
             per_col: int = 8) -> LP:
    """Covering LP A x >= 1 (0/1 matrix) with explicit slacks.

    Columns [0, n) are the structural variables in [0, 1] with integer costs
    in [1, 100]; columns [n, n+m) are the slacks s_i >= 0 with cost 0 and
    coefficient -1 in row i, so the equality form is [A -I][x; s] = 1.  The
    multipliers of the >= rows are bounded below by 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rows, cols = _distinct_rows(rng, m, np.full(n, per_col))
    covered = np.zeros(m, dtype=bool)
    covered[rows] = True
    empty = np.nonzero(~covered)[0].astype(np.uint32)
    if empty.size:
        forced = rng.integers(0, n, size=empty.size).astype(np.uint32)
        rows = np.concatenate([rows, empty])
        cols = np.concatenate([cols, forced])
    vals = np.ones(rows.shape[0])
    srows = np.arange(m, dtype=np.uint32)
    scols = (n + np.arange(m)).astype(np.uint32)
    rows = np.concatenate([rows, srows])
    cols = np.concatenate([cols, scols])
    vals = np.concatenate([vals, -np.ones(m)])
    order = np.lexsort((rows, cols))
    rows, cols, vals = rows[order], cols[order], vals[order]
    cost = rng.integers(1, 101, size=n).astype(np.float32).astype(np.float64)
    linear = np.concatenate([cost, np.zeros(m)])
    lower = np.zeros(n + m)
    upper = np.concatenate([np.ones(n), np.full(m, np.inf)])
    return LP(nrows=m, ncols=n + m, rows=rows, cols=cols, vals=vals,
              rhs=np.ones(m), linear=linear, lower=lower, upper=upper,
              lambda_lower=np.zeros(m), lambda_upper=np.full(m, np.inf),
              name="covering", seed=seed)


def batch_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """m = floor(exp(U[ln lo, ln hi])) for each of `count` instances."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi),
                                       size=count))).astype(np.int64)


def batch_instance(m: int, seed: int, per_col: int = 6) -> LP:
    """One instance of the batched/served workloads: n=2m, 6 nnz/column."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 2 * m
    return _feasible_equality_lp(rng, m, n, np.full(n, per_col), "batch", seed)


def batch(count: int = 512, lo: int = 200, hi: int = 20_000,
          seed: int = 4) -> list[LP]:
    """The batched workload: 512 LPs with m log-uniform in [200, 20,000]."""
    sizes = batch_sizes(count, lo, hi, seed)
    return [batch_instance(int(m), seed * 1_000_003 + i)
            for i, m in enumerate(sizes)]


def stream_schedule(count: int = 20_000, rate: float = 2000.0,
                    lo: int = 500, hi: int = 200_000, seed: int = 5):
    """Arrival times (seconds, Poisson process) and sizes of the served
    stream; instances are built lazily with :func:`batch_instance`."""
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, size=count)
    arrivals = np.cumsum(gaps)
    sizes = batch_sizes(count, lo, hi, seed + 1)
    seeds = seed * 1_000_003 + np.arange(count)
    return arrivals, sizes, seeds


def rel_kkt(lp: LP, x: np.ndarray, lam: np.ndarray) -> dict:
    """Relative KKT residuals of (x, lambda), all in float64.

    primal = ||A x - b||_2 / (1 + ||b||_2)
    dual   = ||x - P[l,u](x - (c - A' lam))||_2 / (1 + ||c||_2)
    gap    = |c'x - (b'lam + sum_j min(l_j r_j, u_j r_j))|
             / (1 + |c'x| + |dual objective|),  r = c - A' lam,
    where a term with an infinite bound and a wrong-sign r_j is left out of
    the dual objective (it is already measured by the dual residual)."""
    r = lp.linear - lp.rmatvec(lam)
    primal = np.linalg.norm(lp.matvec(x) - lp.rhs) / (1 + np.linalg.norm(lp.rhs))
    proj = np.clip(x - r, lp.lower, lp.upper)
    dual = np.linalg.norm(x - proj) / (1 + np.linalg.norm(lp.linear))
    with np.errstate(invalid="ignore", over="ignore"):
        lo_term = np.where(np.isfinite(lp.lower), lp.lower * r, np.inf)
        hi_term = np.where(np.isfinite(lp.upper), lp.upper * r, np.inf)
    lo_term = np.where(np.isfinite(lp.lower) | (r < 0), lo_term, np.inf)
    term = np.minimum(lo_term, hi_term)
    term = np.where(np.isfinite(term), term, 0.0)
    dual_obj = float(lp.rhs @ lam + term.sum())
    pobj = float(lp.linear @ x)
    gap = abs(pobj - dual_obj) / (1 + abs(pobj) + abs(dual_obj))
    return {"primal": float(primal), "dual": float(dual), "gap": float(gap),
            "rel_kkt": float(max(primal, dual, gap)), "objective": pobj}


def write_text(lp: LP, path: str) -> None:
    """Write the plain-text instance format read by alm_read (alm.h:98-117,
    spmv.h:76-83): "nrows ncols nnz", nnz "row col value" triplets, then rhs,
    linear, lower, upper, dual lower, dual upper."""
    def fmt(v):
        return "\n".join("inf" if a == np.inf else "-inf" if a == -np.inf
                         else repr(float(a)) for a in v)
    with open(path, "w") as f:
        f.write(f"{lp.nrows} {lp.ncols} {lp.nnz}\n")
        f.write("\n".join(f"{int(r)} {int(c)} {float(v)!r}" for r, c, v in
                          zip(lp.rows, lp.cols, lp.vals)))
        f.write("\n")
        for v in (lp.rhs, lp.linear, lp.lower, lp.upper, lp.lambda_lower,
                  lp.lambda_upper):
            f.write(fmt(v))
            f.write("\n")
