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
