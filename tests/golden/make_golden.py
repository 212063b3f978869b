"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference compiled from its own sources (oracle/_ref/libacdref.so,
built by ``make -C oracle ref`` where the reference sources exist) on seeded
inputs and stores what it produced.  The inputs are stored too, so the
fixtures do not depend on numpy's generator on the machine that checks them.

    python tests/golden/make_golden.py

Fixtures:
  layouts.npz  small matrices (permuted or not): inputs + SHA-256 of every
               internal layout array the reference built (Z-order COO, CSR
               of A and A', 4-row block offsets and arena bytes, row/column
               permutations) and of the step-size vectors of approx_make.
  small.npz    the 1,000 x 2,000 workload: inputs, the reference ALM+APPROX
               solution (x, lambda, diagnosis, inner iterations, SHA-256 of
               the log), a 3,000-iteration APPROX run from x=0 (x, diagnosis)
               and a 50-iteration mpg_solve run.
"""
from __future__ import annotations

import hashlib
import importlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

inst = importlib.import_module("acd-alm_gb300.instances")

LAYOUT_CASES = [(3, 5, 2, 101), (17, 13, 3, 102), (64, 128, 4, 103),
                (257, 600, 4, 104), (1000, 2000, 5, 105)]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def layout_hashes(lib: O.Lib, lp, permute: bool) -> dict:
    m = lib.matrix(lp, permute)
    lay = lib.layouts(m)
    out = {}
    for key, arrs in lay.items():
        for i, a in enumerate(arrs):
            out[f"{key}.{i}"] = sha(a)
    a = lib.approx(m, lp)
    for p in (0, 1):
        d = lib.internals(a, lp.nrows, lp.ncols, p)
        for k, v in d.items():
            out[f"approx{p}.{k}"] = sha(v)
    lib.approx_free(a)
    lib.matrix_free(m)
    return out


def lp_arrays(lp, prefix: str = "") -> dict:
    return {prefix + k: getattr(lp, k) for k in
            ("rows", "cols", "vals", "rhs", "linear", "lower", "upper",
             "lambda_lower", "lambda_upper")} | {
        prefix + "shape": np.array([lp.nrows, lp.ncols])}


def main() -> None:
    if not O.available("ref"):
        O.build(ref=True)
    ref = O.Lib("ref")
    data = {}
    for idx, (m, n, k, seed) in enumerate(LAYOUT_CASES):
        lp = inst.small(seed=seed, m=m, n=n, per_col=k)
        data.update(lp_arrays(lp, f"c{idx}."))
        for perm in (0, 1):
            for key, h in layout_hashes(ref, lp, bool(perm)).items():
                data[f"c{idx}.p{perm}.{key}"] = np.array(h)
    np.savez_compressed(os.path.join(HERE, "layouts.npz"), **data)

    lp = inst.small()
    out = lp_arrays(lp)
    mat = ref.matrix(lp)
    with tempfile.TemporaryDirectory() as td:
        log = os.path.join(td, "alm.log")
        h = ref.alm(mat, lp)
        r, x, lam, diag, used = ref.alm_solve(h, lp.nrows, lp.ncols, log=log)
        ref.alm_free(h)
        out.update({"alm.ret": np.array(r), "alm.x": x, "alm.lambda": lam,
                    "alm.diag": diag, "alm.inner": np.array(used),
                    "alm.log_sha": np.array(hashlib.sha256(
                        open(log, "rb").read()).hexdigest())})
        a = ref.approx(mat, lp)
        r, x, diag = ref.approx_solve(a, np.zeros(lp.ncols), 3000)
        out.update({"approx.ret": np.array(r), "approx.x": x,
                    "approx.diag": diag})
        r, x, diag = ref.mpg_solve(a, np.zeros(lp.ncols), 50)
        out.update({"mpg.ret": np.array(r), "mpg.x": x, "mpg.diag": diag})
        ref.approx_free(a)
    ref.matrix_free(mat)
    np.savez_compressed(os.path.join(HERE, "small.npz"), **out)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
