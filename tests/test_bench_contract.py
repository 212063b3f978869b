"""bench.py's algorithmic-byte model, checked on CPU against its
definition: per steady-state APPROX iteration, one pass over A and one over
A' (value + column per nonzero) plus the fused epilogues' vector streams,
24 nnz + 4(m+n) + 116 n + 68 m bytes in FP64 and 16 nnz + 4(m+n) + 58 n +
34 m in the mixed form's FP32 iterations (approx.c:343-478 with
gradient_value.inc, step_project.inc and vector.inc)."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Shape:
    def __init__(self, m, n, nnz):
        self.nrows, self.ncols, self.nnz = m, n, nnz


def test_bytes_per_iteration_mid_lp():
    b = _bench()
    lp = _Shape(100_000, 200_000, 2_261_268)
    assert b.bytes_per_iteration(lp, False) == 85_470_432.0
    assert b.bytes_per_iteration(lp, True) == 52_380_288.0


def test_fp32_iteration_moves_fewer_bytes():
    b = _bench()
    for m, n, nnz in ((1, 1, 1), (1000, 2000, 10_000), (10 ** 6, 5 * 10 ** 6, 33 * 10 ** 6)):
        lp = _Shape(m, n, nnz)
        assert b.bytes_per_iteration(lp, True) < b.bytes_per_iteration(lp, False)


def test_reference_arm_line_fits_its_own_run(monkeypatch, capsys, instances):
    """--impl reference: each step is a bounded sample, ms_per_step is that
    sample's measured time (so steps x ms_per_step is the run's length), the
    LPs/s value is a projection whose terms are reported, the precision is
    FP64, and the iterations per LP are the reference's own recorded count."""
    import json
    import sys
    b = _bench()
    monkeypatch.setattr(b, "workload", lambda name: instances.small())
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--workload", "small",
                                      "--steps", "2", "--warmup", "1", "--ref-iters", "300"])
    b.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["dtype"] == "f64"
    assert line["config"]["precision"] == "fp64"
    p = line["projection"]
    assert p["inner_iterations_per_lp"] == 14500  # tests/golden/small_kkt.npz
    assert "small_kkt.npz" in p["source"]
    assert line["ms_per_step"] < 60_000
    assert abs(line["value"] * p["ms_per_iteration"] * 1e-3 * p["inner_iterations_per_lp"]
               - 1.0) < 0.5
    assert line["e2e"]["value"] == line["value"]


def test_auto_precision_threshold_matches_the_library():
    """bench.py resolves --precision auto with the library's own rule
    (mixed_for in csrc/instance.h): the two thresholds must agree."""
    import re
    b = _bench()
    text = open(os.path.join(ROOT, "acd-alm_gb300", "csrc", "instance.h")).read()
    lib_nnz = int(re.search(r"kAutoMixedNnz\s*=\s*(\d+)", text).group(1))
    assert b.AUTO_MIXED_NNZ == lib_nnz
