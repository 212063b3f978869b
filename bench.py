"""Benchmark: LPs solved per second to 1e-6 relative KKT on one GB300.

One step = one LP solved from scratch (x = 0, lambda = 0, unit ALM weights)
by the ALM + APPROX loop until the relative KKT residual is <= 1e-6.
Workload (default): the mid-size LP, m=100,000 rows, n=200,000 columns,
Zipf(1.5) column counts (~2.26M nonzeros), values U[-1,1], box [0,10],
seeded synthetic data.

The headline form is the plain FP64 solve (the drop-in for the reference's
FP64 alm_solve); the FP32 + FP64-refinement form is reported beside it.

Printed (rank 0, one JSON line):
  value         LPs/s from the solve kernel's device time (inputs resident in
                HBM; L2 flushed with a 512 MB write before every step)
  e2e           LPs/s through the C ABI (alm_solve with host arrays: the
                uploads and downloads are inside the timed region)
  roofline      the solve kernel: algorithmic bytes / device time vs the
                measured HBM copy bandwidth
  cpu_baseline  the reference's CPU loop on this host's cores, on a bounded
                sample of the same workload (see `sample`)
  mixed_form    the same LP in the mixed form: LPs/s, iterations, and its
                objective's distance from the FP64 form's and the reference's

  python bench.py [--steps K] [--warmup W] [--precision fp64|mixed]
                  [--workload mid|small] [--impl reference]
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
inst = importlib.import_module("acd-alm_gb300.instances")


def replica_totals(dist, tot_dev: float, tot_wall: float, steps: int, device=None):
    """Whole-job totals of N independent replicas (one LP per rank per step,
    no data-path collective): the time is the slowest rank's, the LPs are
    every rank's.  Returns (LPs, device seconds, wall seconds)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return steps, tot_dev, tot_wall
    import torch
    t = torch.tensor([tot_dev, tot_wall], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    tot_dev, tot_wall = t.tolist()
    return steps * dist.get_world_size(), tot_dev, tot_wall


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name: str):
    if name == "mid":
        return inst.mid()
    if name == "small":
        return inst.small()
    if name == "covering":
        return inst.covering()
    if name in ("batch", "stream"):
        return None
    raise SystemExit(f"unknown workload {name}")


def _plain_fp64_rate(lib, lps):
    """The plain FP64 GPU drop-in, one LP at a time (alm_solve on the whole
    GPU): LPs/s over the given sample, from the solve kernels' device time."""
    tot = 0.0
    for lp in lps:
        m = lib.Matrix(lp)
        a = lib.Alm(m, lp)
        a.set_kkt_tolerance(1e-6)
        a.solve(1000)
        tot += a.stats()["seconds"]
        a.free()
        m.free()
    return len(lps) / tot


def batch_bench(args):
    """--workload batch: the 512-LP batch (m log-uniform in [200, 20000],
    n = 2m, 6 nonzeros per column) in one persistent launch, one LP per CTA,
    to 1e-6 relative KKT; FP64 and mixed forms, each against the plain FP64
    drop-in solving a sample of the same LPs one at a time."""
    lib = importlib.import_module("acd-alm_gb300.lib")
    lps = inst.batch(args.batch_count)
    mats = [lib.Matrix(lp) for lp in lps]
    alms = [lib.Alm(m, lp) for m, lp in zip(mats, lps)]
    L = lib.lib()
    forms = []
    for prec, name in ((0, "fp64"), (1, "mixed")):
        for a, lp in zip(alms, lps):
            a.set_kkt_tolerance(1e-6)
            a.set_precision(prec)
            w = np.ctypeslib.as_array(L.approx_weight(L.acdalm_alm_approx(a.h)), (lp.nrows,))
            w[:] = 1.0
        b = lib.Batch(alms)
        ret, xs, lams, diag = b.solve(1000)
        sec = b.seconds()
        kk = [inst.rel_kkt(lps[i], xs[i], lams[i])["rel_kkt"]
              for i in range(0, len(lps), max(1, len(lps) // 16))]
        forms.append({"precision": name, "value": len(lps) / sec, "device_s": sec,
                      "solved": int((ret == 0).sum()), "rel_kkt_host_sample_max": max(kk)})
        b.free()
    sample = [lps[i] for i in range(0, len(lps), max(1, len(lps) // args.plain_sample))]
    plain = _plain_fp64_rate(lib, sample)
    for a in alms:
        a.free()
    for m in mats:
        m.free()
    best = max(forms, key=lambda f: f["value"])
    print(json.dumps({"metric": "LPs/sec to 1e-6 relative KKT (batch)", "value": best["value"],
                      "unit": "LP/s", "n_gpus": 1, "higher_is_better": True,
                      "dtype": "f64" if best["precision"] == "fp64" else "f32+f64",
                      "data": "synthetic",
                      "config": {"workload": f"batch of {len(lps)} LPs",
                                 "m": "log-uniform [200, 20000]", "n": "2m",
                                 "nnz_total": int(sum(lp.nnz for lp in lps))},
                      "forms": forms,
                      "plain_fp64_one_at_a_time": {"value": plain, "sample": len(sample)},
                      "vs_plain_fp64": best["value"] / plain}), flush=True)


def stream_bench(args):
    """--workload stream: the first --stream-count requests of the served
    stream (m log-uniform in [500, 200000], Poisson arrivals at 2000/s)
    through the continuous-batching server; LPs/s over the wall time from
    the first arrival to the last result, p50 / p99 latency (submission to
    completion), against the plain FP64 drop-in one at a time on a sample."""
    import threading
    lib = importlib.import_module("acd-alm_gb300.lib")
    arrivals, sizes, seeds = inst.stream_schedule()
    k = args.stream_count
    arrivals, sizes, seeds = arrivals[:k], sizes[:k], seeds[:k]
    lps = [inst.batch_instance(int(m), int(sd)) for m, sd in zip(sizes, seeds)]
    prec = {"fp64": 0, "mixed": 1, "auto": 2}[args.precision]
    srv = lib.Server(precision=prec, kkt_tol=1e-6)
    t0 = time.perf_counter()
    sub = {}

    def submitter():
        for i, lp in enumerate(lps):
            now = time.perf_counter() - t0
            if arrivals[i] > now:
                time.sleep(arrivals[i] - now)
            sub[srv.submit(lp)] = i

    th = threading.Thread(target=submitter)
    th.start()
    done = {}
    while len(done) < k and time.perf_counter() - t0 < args.stream_limit:
        for rid in srv.poll(timeout=0.5):
            done[rid] = srv.result(rid)
    wall = time.perf_counter() - t0
    th.join()
    srv.close()
    lat = np.array([v[4] for v in done.values()])
    msz = np.array([int(sizes[sub[r]]) for r in done if r in sub])
    lat_m = np.array([done[r][4] for r in done if r in sub])
    by_m = {}
    for name, sel in (("m<=20000", msz <= 20000), ("m>20000", msz > 20000)):
        if sel.any():
            by_m[name] = {"count": int(sel.sum()), "p50_s": float(np.percentile(lat_m[sel], 50)),
                          "p99_s": float(np.percentile(lat_m[sel], 99))}
    kk = [v[3]["rel_kkt"] for v in done.values()]
    sample = [lps[i] for i in range(0, k, max(1, k // args.plain_sample))]
    plain = _plain_fp64_rate(lib, sample)
    rate = len(done) / wall
    print(json.dumps({"metric": "LPs/sec and p50/p99 latency to 1e-6 relative KKT (stream)",
                      "value": rate, "unit": "LP/s", "n_gpus": 1, "higher_is_better": True,
                      "dtype": "f64" if prec == 0 else "f32+f64", "data": "synthetic",
                      "config": {"workload": f"first {k} requests of the served stream",
                                 "m": "log-uniform [500, 200000]", "n": "2m",
                                 "arrivals": "Poisson 2000/s", "max_m": int(sizes.max())},
                      "completed": len(done), "solved": sum(1 for v in done.values() if v[0] == 0),
                      "arrival_span_s": float(arrivals[-1]) if k else 0.0,
                      "latency_by_size": by_m,
                      "requests": k, "precision": args.precision,
                      "wall_s": wall, "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
                      "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
                      "rel_kkt_device_max": max(kk) if kk else None,
                      "plain_fp64_one_at_a_time": {"value": plain, "sample": len(sample)},
                      "vs_plain_fp64": rate / plain}), flush=True)


def cusparse_comparator(lp, reps, flush, peak):
    """The library comparator for the SpMV kernels: cuSPARSE's CSR product
    through torch's sparse CSR matmul (one right-hand side), y = A x and
    y = A'x in FP64 and FP32, with the same L2 flush and byte model."""
    import scipy.sparse as sp
    import torch
    out = []
    try:
        a = sp.csr_matrix((lp.vals, (lp.rows, lp.cols)), shape=(lp.nrows, lp.ncols))
        for t, mat in ((0, a), (1, a.T.tocsr())):
            for dt in (torch.float64, torch.float32):
                op = torch.sparse_csr_tensor(
                    torch.from_numpy(mat.indptr.astype(np.int32)).cuda(),
                    torch.from_numpy(mat.indices.astype(np.int32)).cuda(),
                    torch.from_numpy(mat.data).to(dt).cuda(), size=mat.shape)
                x = torch.rand(mat.shape[1], 1, dtype=dt, device="cuda")
                for _ in range(3):
                    y = op @ x
                stream = torch.cuda.current_stream()
                times = []
                for _ in range(reps):
                    flush.fill_(1.0)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    y = op @ x
                    e1.record(stream)
                    torch.cuda.synchronize()
                    times.append(e0.elapsed_time(e1) * 1e-3)
                sec = statistics.median(times)
                sv = 4 if dt == torch.float32 else 8
                ny, nx = mat.shape
                nbytes = lp.nnz * (sv + 4) + 4 * (ny + 1) + sv * (nx + ny)
                out.append({"variant": "cusparse_csr", "op": "A'x" if t else "Ax",
                            "dtype": "f32" if sv == 4 else "f64", "us": round(sec * 1e6, 1),
                            "gbs": round(nbytes / sec / 1e9, 1),
                            "frac": round(nbytes / sec / 1e9 / peak, 3)})
                del op, x, y
    except Exception as e:  # the comparator is reported, never required
        out.append({"variant": "cusparse_csr", "error": str(e)[:200]})
    return out


def served_probe(args):
    """--served M --profile-solve N: one LP of the served-stream family
    (m = M, n = 2m, 6 nonzeros per column) alone in a server, capped at N
    inner iterations (the command the ncu captures of the one-CTA and
    cluster kernels use)."""
    lib = importlib.import_module("acd-alm_gb300.lib")
    lp = inst.batch_instance(args.served, 12345 + args.served)
    prec = {"fp64": 0, "mixed": 1, "auto": 2}[args.precision]
    srv = lib.Server(precision=prec, kkt_tol=1e-6)
    srv.set_inner_budget(args.profile_solve)
    srv.submit(lp)
    got = []
    while not got:
        got = srv.poll(timeout=1.0)
    r, x, lam, st, lat = srv.result(got[0])
    srv.close()
    print(json.dumps({"served": args.served, "nnz": lp.nnz, "precision": args.precision,
                      "profile_solve": args.profile_solve, "ret": r,
                      "inner": st["inner_iterations"], "device_seconds": st["seconds"]}))


def spmv_bench(args, lp):
    """--spmv: y = A x and y = A'x on the device, every layout variant, FP64
    and FP32, L2 flushed before each timed launch; GB/s from the algorithmic
    bytes nnz*(value+4) + 4*(rows+1) + value*(rows+cols)."""
    import torch
    lib = importlib.import_module("acd-alm_gb300.lib")
    L = lib.lib()
    m = lib.Matrix(lp)
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    peak, peak_kind = load_peaks()
    names = {0: "sell", 1: "block", 2: "csr", 3: "sell_fma"}
    out = []
    for variant in (0, 3, 2, 1):
        for t in (0, 1):
            for f32 in (False, True):
                if variant in (1, 3) and f32:
                    continue
                dt = torch.float32 if f32 else torch.float64
                nx, ny = (lp.nrows, lp.ncols) if t else (lp.ncols, lp.nrows)
                x = torch.rand(nx, dtype=dt, device="cuda")
                y = torch.empty(ny, dtype=dt, device="cuda")
                fn = L.acdalm_spmv_device_f32 if f32 else L.acdalm_spmv_device
                for _ in range(3):
                    lib.check(fn(m.h, variant, t, x.data_ptr(), y.data_ptr(), stream.cuda_stream),
                              "spmv")
                times = []
                for _ in range(args.spmv_reps):
                    flush.fill_(1.0)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    fn(m.h, variant, t, x.data_ptr(), y.data_ptr(), stream.cuda_stream)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    times.append(e0.elapsed_time(e1) * 1e-3)
                sec = statistics.median(times)
                sv = 4 if f32 else 8
                nbytes = lp.nnz * (sv + 4) + 4 * (ny + 1) + sv * (nx + ny)
                out.append({"variant": names[variant], "op": "A'x" if t else "Ax",
                            "dtype": "f32" if f32 else "f64", "us": round(sec * 1e6, 1),
                            "gbs": round(nbytes / sec / 1e9, 1),
                            "frac": round(nbytes / sec / 1e9 / peak, 3),
                            "exact": (not f32) and variant in (0, 1)})
    best = max(out, key=lambda r: r["gbs"])
    line = {"metric": "SpMV HBM GB/s (covering LP)", "value": best["gbs"], "unit": "GB/s",
            "n_gpus": 1, "steps": args.spmv_reps, "warmup": 3,
            "ms_per_step": best["us"] / 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": best["dtype"], "data": "synthetic",
            "config": {"workload": "covering LP", "m": lp.nrows, "n": lp.ncols, "nnz": lp.nnz,
                       "l2": "flushed (512 MB write) before every launch"},
            "roofline": {"bound": "hbm", "achieved": best["gbs"], "peak": peak, "unit": "GB/s",
                         "frac": best["gbs"] / peak, "traffic": None,
                         "kernel": f"{best['variant']} {best['op']} {best['dtype']}",
                         "peak_source": peak_kind},
            "variants": out,
            "library_comparator": cusparse_comparator(lp, args.spmv_reps, flush, peak)}
    print(json.dumps(line), flush=True)
    m.free()


def layout_bench(args, lp):
    """--layout: the reference's layouts of the workload's matrix (row and
    column nonzero-count permutations, CSR of A and A' of the permuted
    matrix: what approx_make's shadow copy holds) built on the host
    (sparse_matrix_make with permute = 1) and on the GPU
    (acdalm_layout_device, triplets resident in HBM), best of --spmv-reps."""
    import ctypes
    import torch
    lib = importlib.import_module("acd-alm_gb300.lib")
    L = lib.lib()
    f = L.acdalm_layout_device
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_size_t] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_int] \
        + [ctypes.c_void_p] * 9
    host = []
    for _ in range(min(3, args.spmv_reps)):
        t0 = time.perf_counter()
        mm = lib.Matrix(lp, permute=True)
        host.append(time.perf_counter() - t0)
        mm.free()
    i32 = lambda a: torch.tensor(np.ascontiguousarray(a, np.uint32).view(np.int32), device="cuda")
    rows, cols = i32(lp.rows), i32(lp.cols)
    vals = torch.tensor(np.ascontiguousarray(lp.vals), device="cuda")
    z = lambda k, dt=torch.int32: torch.empty(max(k, 1), dtype=dt, device="cuda")
    outs = [z(lp.nrows), z(lp.ncols), z(lp.nrows + 1), z(lp.nnz), z(lp.nnz, torch.float64),
            z(lp.ncols + 1), z(lp.nnz), z(lp.nnz, torch.float64)]
    stream = torch.cuda.current_stream()
    dev = []
    for rep in range(args.spmv_reps + 1):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = f(lp.nrows, lp.ncols, lp.nnz, rows.data_ptr(), cols.data_ptr(), vals.data_ptr(), 1,
              *[o.data_ptr() for o in outs], stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        lib.check(r, "acdalm_layout_device")
        if rep:
            dev.append(e0.elapsed_time(e1) * 1e-3)
    print(json.dumps({"metric": "layout build seconds (permutations + CSR of A and A')",
                      "workload": args.workload, "m": lp.nrows, "n": lp.ncols, "nnz": lp.nnz,
                      "host_s": min(host), "gpu_s": min(dev), "speedup": min(host) / min(dev),
                      "host_note": "sparse_matrix_make(permute=1) on one host thread",
                      "gpu_note": "acdalm_layout_device, triplets resident, CUDA events"}),
          flush=True)


def bytes_per_iteration(lp, fp32: bool) -> float:
    """Algorithmic bytes of one steady-state APPROX iteration: one pass over
    A and one over A' (each nonzero's value and column read once), plus the
    vector streams of the fused epilogues."""
    nnz, m, n = lp.nnz, lp.nrows, lp.ncols
    if fp32:
        return 16.0 * nnz + 4.0 * (m + n) + 58.0 * n + 34.0 * m
    return 24.0 * nnz + 4.0 * (m + n) + 116.0 * n + 68.0 * m


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "samples": len(rows), "reasons": sorted(reasons)}


GOLDEN = os.path.join(ROOT, "tests", "golden")


def reference_solve_record(workload: str):
    """The reference's own solve of this workload to relative KKT <= 1e-6
    (inner iterations, objective), recorded by running the reference
    compiled from its sources (tests/golden/make_kkt_golden.py): the
    iterations a CPU solve of this LP takes.  None if not recorded."""
    name = {"mid": "mid.npz", "small": "small_kkt.npz"}.get(workload)
    path = os.path.join(GOLDEN, name) if name else None
    if not path or not os.path.exists(path):
        return None
    g = np.load(path)
    return {"inner_iterations": int(g["inner"]), "outer_iterations": int(g["outer"]),
            "objective": float(g["objective"]), "rel_kkt": float(g["host_kkt"][3]),
            "source": f"tests/golden/{name}"}


def cpu_baseline(lp, inner_per_lp: float, iters: int, threads: int, per_lp_source: str):
    """The reference's inner loop on the host cores, over a bounded sample:
    `iters` APPROX iterations on the same LP (the loop that dominates a
    solve: ~23 outer vs ~10^5 inner iterations), one ALM outer iteration's
    set-up included; LPs/s is projected with `inner_per_lp` inner
    iterations per LP (the reference's own count for this LP where it was
    recorded)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    kind = "reference" if O.available("ref") else "port"
    if kind == "port" and not O.available("oracle"):
        O.build(ref=False)
    lib = O.Lib("ref" if kind == "reference" else "oracle")
    m = lib.matrix(lp)
    a = lib.approx(m, lp)
    x0 = np.zeros(lp.ncols)
    t0 = time.perf_counter()
    r, x, diag = lib.approx_solve(a, x0, iters, max_pg=0.0, threads=threads)
    dt = time.perf_counter() - t0
    lib.approx_free(a)
    lib.matrix_free(m)
    # iterations actually run (diag[4], approx.c:681-702); min_delta = 0 and
    # max_pg = 0 keep the loop going, this guards an early exit
    done = int(diag[4]) if diag[4] > 0 else iters
    iters = min(iters, done)
    per_iter = dt / max(iters, 1)
    return {"value": 1.0 / (per_iter * inner_per_lp), "unit": "LP/s",
            "cores": threads, "kind": kind,
            "sample": (f"{iters} APPROX iterations of the same LP on {threads} threads "
                       f"({dt:.1f} s, {per_iter * 1e3:.3f} ms/iteration), projected to "
                       f"{inner_per_lp:.0f} inner iterations per LP ({per_lp_source}; the "
                       f"outer ALM work is <1% of a solve)"),
            "sample_seconds": dt, "sample_iterations": iters,
            "ms_per_iteration": per_iter * 1e3, "inner_iterations_per_lp": inner_per_lp}


def inner_per_lp_of(args, fallback=None):
    """Inner iterations per LP for the CPU projection: the reference's own
    count for this workload where recorded, else `fallback` (the GPU FP64
    solve's count), else a round figure.  Returns (count, source)."""
    rec = reference_solve_record(args.workload)
    if rec:
        return float(rec["inner_iterations"]), (
            f"the reference's own count for this LP, {rec['source']}")
    if fallback:
        return float(fallback), "the FP64 GPU solve's count for the same LP"
    return 100000.0, "a round figure: no recorded count for this workload"


def run_reference(args, lp, rank: int):
    """--impl reference: the reference's CPU implementation of the loop on
    the host cores (oracle/_ref where it was compiled, else the oracle port),
    each step a bounded sample of the workload: --ref-iters APPROX
    iterations.  ms_per_step is that sample's time; value (LPs/s) projects
    the sample's time per iteration to the reference's own iterations per
    LP, and the projection's terms are in `projection`."""
    threads = os.cpu_count() or 1
    per_lp, source = inner_per_lp_of(args)
    vals, secs = [], []
    base = None
    for s in range(args.warmup + args.steps):
        base = cpu_baseline(lp, per_lp, args.ref_iters, threads, source)
        if s >= args.warmup:
            vals.append(base["value"])
            secs.append(base["sample_seconds"])
    v = statistics.median(vals)
    base["value"] = v
    cfg = config_of(args, lp)
    cfg["precision"] = "fp64"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "LP/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "cpu_baseline": base,
            "projection": {"ms_per_iteration": base["ms_per_iteration"],
                           "inner_iterations_per_lp": per_lp, "source": source,
                           "seconds_per_lp": 1.0 / v,
                           "step": f"{args.ref_iters} APPROX iterations (a bounded sample)"},
            "e2e": {"value": v, "unit": "LP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if rank == 0:
        print(json.dumps(line), flush=True)


METRIC = "LPs/sec to 1e-6 relative KKT"
# ACDALM_PRECISION_AUTO runs FP32 inner iterations from this many nonzeros on
AUTO_MIXED_NNZ = 500_000

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one FP64 inner
# iteration of the mid LP's solve kernel, from one ncu capture of
# `bench.py --profile-solve 3000` (3,000 FP64 iterations;
# profiles/alm_kernel_mid_traffic.md).  FP32 iterations are scaled by their
# algorithmic bytes.
MID_DRAM_BYTES_PER_FP64_ITER = (27516251648 + 10049832192) / 3000
TRAFFIC_NOTE = ("ncu DRAM bytes per launch, scaled from a 3,000-iteration capture of the "
                "same kernel; the instance stays in L2, so traffic is far below the "
                "algorithmic bytes")


def config_of(args, lp):
    return {"workload": f"{args.workload} LP", "m": lp.nrows, "n": lp.ncols, "nnz": lp.nnz,
            "stop": "relative KKT <= 1e-6 (max of primal, dual, gap)",
            "precision": args.precision, "l2": "flushed (512 MB write) before every step",
            "seed": lp.seed}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="mid")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed", "auto"],
                    help="the headline form (fp64: the reference's arithmetic)")
    ap.add_argument("--profile-solve", type=int, default=0,
                    help="run one ALM solve capped at this many inner iterations and exit "
                         "(the command the ncu captures use)")
    ap.add_argument("--served", type=int, default=0,
                    help="with --profile-solve: serve one LP of the served-stream family "
                         "with this many rows instead (one CTA or a cluster, as the server "
                         "picks), capped the same way")
    ap.add_argument("--trace", type=int, default=0,
                    help="trace this many grid-team reductions (from the 2,001st) of one "
                         "solve capped at 3,000 inner iterations; print the phase breakdown")
    ap.add_argument("--ref-iters", type=int, default=4000,
                    help="APPROX iterations each CPU sample times (about 6 s on 16 cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default layout instead of acdalm_autotune's choice")
    ap.add_argument("--side-steps", type=int, default=2,
                    help="solves of the other precision form, reported beside the "
                         "headline (0 = none)")
    ap.add_argument("--spmv", action="store_true",
                    help="time the device SpMV variants on the workload's matrix")
    ap.add_argument("--spmv-reps", type=int, default=10)
    ap.add_argument("--layout", action="store_true",
                    help="time the layout build (host vs GPU) on the workload's matrix")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--stream-count", type=int, default=48)
    ap.add_argument("--stream-limit", type=float, default=900.0,
                    help="seconds after which the stream run stops collecting")
    ap.add_argument("--plain-sample", type=int, default=8,
                    help="LPs the plain FP64 comparison solves one at a time")
    args = ap.parse_args()
    if args.precision is None:
        # the served stream runs the library's size rule; single LPs the
        # FP64 drop-in
        args.precision = "auto" if args.workload == "stream" else "fp64"
    if args.served and args.profile_solve:
        served_probe(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    lp = workload(args.workload)
    if lp is not None and args.precision == "auto":
        # ACDALM_PRECISION_AUTO's rule, resolved for this one LP
        args.precision = "mixed" if lp.nnz >= AUTO_MIXED_NNZ else "fp64"

    if args.impl == "reference":
        if rank == 0:
            if lp is None:
                print(json.dumps({"impl": "reference",
                                  "unavailable": "the CPU arm times single-LP workloads "
                                                 "(mid, small, covering) only"}), flush=True)
            else:
                run_reference(args, lp, rank)
        return

    if args.spmv:
        spmv_bench(args, lp)
        return
    if args.layout:
        layout_bench(args, lp)
        return
    if args.workload == "batch":
        batch_bench(args)
        return
    if args.workload == "stream":
        stream_bench(args)
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    os.environ.setdefault("ACDALM_DEVICE", str(local))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    lib = importlib.import_module("acd-alm_gb300.lib")
    L = lib.lib()
    if args.trace:
        trace_solve(args, lib, lp)
        return
    if args.profile_solve:
        m = lib.Matrix(lp)
        alm = lib.Alm(m, lp)
        if args.precision == "mixed":
            alm.set_precision(lib.PRECISION_MIXED)
        alm.set_inner_budget(args.profile_solve)
        alm.solve(1000)
        st = alm.stats()
        print(json.dumps({"profile_solve": args.profile_solve, "workload": args.workload,
                          "precision": args.precision, "inner": st["inner_iterations"],
                          "inner32": st["fp32_inner_iterations"],
                          "device_seconds": st["seconds"]}))
        return
    L.acdalm_launch_count.restype = __import__("ctypes").c_ulonglong
    m = lib.Matrix(lp)
    alm = lib.Alm(m, lp)
    # the layout's step cap, picked by timing on this GPU (untimed set-up)
    tuned = alm.autotune(300) if not args.no_autotune else None
    alm.set_kkt_tolerance(1e-6)
    if args.precision == "mixed":
        alm.set_precision(lib.PRECISION_MIXED)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    weights = np.ctypeslib.as_array(_alm_weight(L, alm), (lp.nrows,))

    def reset_state():
        # unit ALM weights: each step starts the same solve from scratch
        weights[:] = 1.0

    def one_step():
        reset_state()
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r, x, lam, diag = alm.solve(1000)
        t1 = time.perf_counter()
        st = alm.stats()
        return r, x, lam, st, t1 - t0

    for _ in range(args.warmup):
        one_step()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    launches0 = L.acdalm_launch_count()
    dev_s, wall_s, inner, outer, kkts, inner32 = [], [], [], [], [], []
    for _ in range(args.steps):
        r, x, lam, st, wall = one_step()
        dev_s.append(st["seconds"])
        wall_s.append(wall)
        inner.append(st["inner_iterations"])
        inner32.append(st["fp32_inner_iterations"])
        outer.append(st["outer_iterations"])
        kkts.append(st["rel_kkt"])
    torch.cuda.synchronize()
    launches = L.acdalm_launch_count() - launches0
    clk = clocks.stop()
    n_lp, tot_dev, tot_wall = replica_totals(dist, sum(dev_s), sum(wall_s), args.steps,
                                             device="cuda")
    value = n_lp / tot_dev
    e2e = n_lp / tot_wall
    k = inst.rel_kkt(lp, x, lam)
    fp32 = args.precision == "mixed"
    ref_rec = reference_solve_record(args.workload)
    side = None
    if args.side_steps > 0:
        # the other precision form of the same solve, for comparison
        other = "fp64" if fp32 else "mixed"
        alm.set_precision(lib.PRECISION_FP64 if fp32 else lib.PRECISION_MIXED)
        sides = [one_step() for _ in range(args.side_steps)]
        alm.set_precision(lib.PRECISION_MIXED if fp32 else lib.PRECISION_FP64)
        r2, x2, l2, st2, _ = sides[-1]
        k2 = inst.rel_kkt(lp, x2, l2)
        sec2 = statistics.median(s_[3]["seconds"] for s_ in sides)
        side = {"precision": other, "value": 1.0 / sec2, "unit": "LP/s",
                "device_seconds": [s_[3]["seconds"] for s_ in sides],
                "inner_iterations": st2["inner_iterations"],
                "fp32_inner_iterations": st2["fp32_inner_iterations"],
                "rel_kkt_host_check": k2["rel_kkt"], "objective": k2["objective"],
                "objective_rel_diff_vs_headline":
                    abs(k2["objective"] - k["objective"]) / abs(k["objective"])}
        if ref_rec:
            side["objective_rel_diff_vs_reference"] = (
                abs(k2["objective"] - ref_rec["objective"]) / abs(ref_rec["objective"]))
    bpi = bytes_per_iteration(lp, False)
    bpi32 = bytes_per_iteration(lp, True)
    mean_inner = float(np.mean(inner))
    mean_inner32 = float(np.mean(inner32))
    # FP32 iterations move 16 B per nonzero, FP64 ones 24 B
    algo_bytes = mean_inner32 * bpi32 + (mean_inner - mean_inner32) * bpi
    achieved = algo_bytes / (tot_dev / args.steps) / 1e9
    peak, peak_kind = load_peaks()
    traffic = None
    if args.workload == "mid":
        traffic = (MID_DRAM_BYTES_PER_FP64_ITER * (mean_inner - mean_inner32)
                   + MID_DRAM_BYTES_PER_FP64_ITER * bpi32 / bpi * mean_inner32)
    line = {
        "metric": METRIC, "value": value, "unit": "LP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if fp32 else "f64", "data": "synthetic",
        "config": config_of(args, lp),
        "e2e": {"value": e2e, "unit": "LP/s",
                "h2d_bytes_per_step": 8 * (3 * lp.nrows + 4 * lp.ncols + lp.nrows + lp.ncols),
                "d2h_bytes_per_step": 8 * (2 * lp.ncols + 2 * lp.nrows)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "traffic_note": TRAFFIC_NOTE if traffic is not None
                     else "no ncu DRAM capture of this workload",
                     "kernel": "alm_kernel (persistent cooperative solve)",
                     "peak_source": peak_kind,
                     "bytes_per_inner_iteration": {"fp64": bpi, "fp32": bpi32}},
        "gpu_launches": int(launches),
        ("fp64_form" if fp32 else "mixed_form"): side,
        "solve": {"inner_iterations": inner, "fp32_inner_iterations": inner32,
                  "outer_iterations": outer,
                  "rel_kkt_device": kkts, "rel_kkt_host_check": k["rel_kkt"],
                  "objective": k["objective"], "device_seconds": dev_s,
                  "wall_seconds": wall_s},
        "reference_solve": ref_rec,
        "layout": {"max_steps": tuned, "chosen_by": "acdalm_autotune (300 APPROX iterations "
                   "per candidate cap, before the warm-up)" if tuned is not None else "default"},
        "clocks": clk,
    }
    if ref_rec:
        line["solve"]["objective_rel_diff_vs_reference"] = (
            abs(k["objective"] - ref_rec["objective"]) / abs(ref_rec["objective"]))
    if rank == 0 and not args.no_cpu_baseline:
        per_lp, source = inner_per_lp_of(args, fallback=mean_inner if not fp32 else None)
        line["cpu_baseline"] = cpu_baseline(lp, per_lp, args.ref_iters,
                                            os.cpu_count() or 1, source)
        # the same loop on one thread (a shorter sample)
        one = cpu_baseline(lp, per_lp, max(200, args.ref_iters // 16), 1, source)
        line["cpu_baseline"]["single_thread"] = {
            k: one[k] for k in ("value", "cores", "sample", "ms_per_iteration")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    alm.free()
    m.free()
    if dist:
        dist.destroy_process_group()


def trace_solve(args, lib, lp, first=2001):
    """--trace N: one solve of the workload capped at 3,000 inner iterations,
    with the grid team's reductions first .. first + N - 1 traced (two per
    steady-state inner iteration: the A' pass and the A pass); prints where
    the time of an iteration goes.  Times in ns, from %globaltimer."""
    m = lib.Matrix(lp)
    alm = lib.Alm(m, lp)
    if args.precision == "mixed":
        alm.set_precision(lib.PRECISION_MIXED)
    alm.set_inner_budget(3000)
    alm.set_trace(first, args.trace)
    alm.solve(1000)
    st = alm.stats()
    t = alm.trace().astype(np.int64)          # [reduction, cta, phase]
    alm.free()
    m.free()
    ok = (t > 0).all(axis=(1, 2))
    es = [e for e in range(1, t.shape[0]) if ok[e] and ok[e - 1]]
    enter, ready, leave = t[:, :, 0], t[:, :, 1], t[:, :, 2]
    pas = np.array([enter[e] - leave[e - 1] for e in es])       # per CTA: its warp 0's pass
    whole = np.array([ready[e] - leave[e - 1] for e in es])     # per CTA: the CTA's pass
    last = np.array([ready[e].max() for e in es])
    after = np.array([leave[e] - last[i] for i, e in enumerate(es)])
    blk = np.array([ready[e] - enter[e] for e in es])
    cycle = np.array([leave[e].max() - leave[e - 1].max() for e in es])

    def st_(a):
        return {"mean": float(a.mean()), "p50": float(np.median(a)), "max": float(a.max())}

    out = {"trace": args.trace, "workload": args.workload, "precision": args.precision,
           "ctas": int(t.shape[1]), "inner_iterations": st["inner_iterations"],
           "us_per_inner_iteration": st["seconds"] / max(st["inner_iterations"], 1) * 1e6,
           "reduction_cycle_ns": st_(cycle),
           "cta_pass_ns": {"mean_over_ctas": st_(whole.mean(1)), "max_over_ctas": st_(whole.max(1))},
           "warp0_pass_ns": st_(pas), "block_reduce_ns": st_(blk),
           "leave_after_last_cta_ready_ns": st_(after)}
    for par in (0, 1):
        sel = [i for i, e in enumerate(es) if (e + first) % 2 == par]
        if sel:
            out[f"reductions_{par}_mod_2"] = {"cycle": st_(cycle[sel]),
                                              "cta_pass_max": st_(whole[sel].max(1)),
                                              "cta_pass_mean": st_(whole[sel].mean(1))}
    slow = whole.mean(0)
    out["slowest_ctas"] = [int(i) for i in np.argsort(-slow)[:8]]
    out["cta_pass_mean_ns_by_cta"] = {"max": float(slow.max()), "min": float(slow.min())}
    print(json.dumps(out), flush=True)


def _alm_weight(L, alm):
    """The ALM instance's weight vector (approx_weight of its APPROX)."""
    import ctypes
    L.acdalm_alm_approx.restype = ctypes.c_void_p
    L.acdalm_alm_approx.argtypes = [ctypes.c_void_p]
    a = L.acdalm_alm_approx(alm.h)
    return L.approx_weight(a)


if __name__ == "__main__":
    main()
