"""Generate tests/golden/small_kkt.npz and tests/golden/mid.npz from the
reference itself.

Runs the reference compiled from its own sources (oracle/_ref/libacdref.so,
built by ``make -C oracle ref`` where the reference sources exist): its
alm_solve (alm.c:289-322) over its own APPROX (approx/approx.c:576-708,
reached through ref_shim.c's cd_solve forwarder), stopped at relative KKT
<= 1e-6 checked at the start of every outer iteration after the first
(ref_alm_solve_kkt) -- the stop rule the benchmark's metric uses.  One
thread by default, so the runs are bit-reproducible.

  small_kkt.npz  the 1,000 x 2,000 workload (seed 1, 5 nonzeros per column);
                 about a second.
  covering_kkt.npz  a reduced covering LP (A x >= 1 with slacks, m = 5,000,
                 n = 20,000 + 5,000 slacks, 8 ones per column, seed 3).
  mid.npz        the mid-size LP (m = 100,000, n = 200,000, Zipf(1.5) column
                 counts, 2,261,268 nonzeros, seed 2); about half an hour on
                 one x86 core.

The instances are regenerated from their seeds by the tests; their SHA-256
is stored, so a test can tell that it rebuilt the same LP.

    python tests/golden/make_kkt_golden.py [small|covering|mid|all] [--threads N]

Each file holds: shape (m, n, nnz), instance_sha256, seed, tol, ret,
kkt (primal, dual, gap and c'x at the stop, as the shim computed them),
host_kkt (primal, dual, gap, max from instances.rel_kkt on the returned x
and lambda), objective (c'x), outer and inner iteration counts, seconds,
threads.
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

inst = importlib.import_module("acd-alm_gb300.instances")

WORKLOADS = {"small": ("small_kkt.npz", inst.small), "mid": ("mid.npz", inst.mid),
             "covering": ("covering_kkt.npz", lambda: inst.covering(m=5000, n=20000))}


def run(ref: O.Lib, lp, tol: float, threads: int, out: str) -> None:
    m = ref.matrix(lp)
    h = ref.alm(m, lp)
    t0 = time.perf_counter()
    ret, x, lam, kk, outer, inner = ref.alm_solve_kkt(h, lp.nrows, lp.ncols, tol,
                                                      threads=threads)
    sec = time.perf_counter() - t0
    host = inst.rel_kkt(lp, x, lam)
    ref.alm_free(h)
    ref.matrix_free(m)
    np.savez(out, shape=np.array([lp.nrows, lp.ncols, lp.nnz]),
             instance_sha256=np.array(lp.sha256()), seed=np.array(lp.seed),
             tol=np.array(tol), ret=np.array(ret), kkt=kk,
             host_kkt=np.array([host["primal"], host["dual"], host["gap"], host["rel_kkt"]]),
             objective=np.array(host["objective"]), outer=np.array(outer),
             inner=np.array(inner), seconds=np.array(sec), threads=np.array(threads))
    print(f"{os.path.basename(out)}: ret {ret}, objective {host['objective']:.12g}, "
          f"rel-KKT {host['rel_kkt']:.3e} (shim {max(kk[:3]):.3e}), {outer} outer / "
          f"{inner} inner iterations, {sec:.1f} s on {threads} thread(s)", flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="?", default="all",
                    choices=["small", "mid", "covering", "all"])
    ap.add_argument("--threads", type=int, default=1)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--outdir", default=HERE)
    args = ap.parse_args()
    if not O.available("ref"):
        O.build(ref=True)
    ref = O.Lib("ref")
    names = ["small", "covering", "mid"] if args.which == "all" else [args.which]
    for name in names:
        fname, make = WORKLOADS[name]
        run(ref, make(), args.tol, args.threads, os.path.join(args.outdir, fname))


if __name__ == "__main__":
    main()
