"""acdalm_read_mps: a free-format MPS LP in the solver's form (slack columns
for inequality and ranged rows, free multipliers), checked entry by entry
and by solving it with the oracle (the reference's ALM restated) on the
CPU.  Host-only: no GPU needed."""
import ctypes

import numpy as np
import pytest

from libutil import binding

libc = ctypes.CDLL(None)
libc.fopen.restype = ctypes.c_void_p
libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
libc.fclose.argtypes = [ctypes.c_void_p]

# min -3x - 2y + z  s.t.  x + y <= 4,  x + 3y <= 6,  -2 <= z - y <= 3,
# x + z = 4,  0 <= x <= 3,  y >= 0,  z free.  With z = 4 - x the objective
# is 4 - 4x - 2y, minimised at x = 3, y = 1 (z = 1): -10.
LP_MPS = """NAME          TINY
* a comment line
ROWS
 N  COST
 L  C1
 L  C2
 G  C3
 E  C4
COLUMNS
    X  COST  -3.0  C1  1.0
    X  C2    1.0   C4  1.0
    Y  COST  -2.0  C1  1.0
    Y  C2    3.0   C3  -1.0
    MARKER  'MARKER'  'INTORG'
    Z  COST  1.0   C3  1.0
    Z  C4    1.0
    MARKER  'MARKER'  'INTEND'
RHS
    RHS  C1  4.0   C2  6.0
    RHS  C3  -2.0  C4  4.0
RANGES
    RNG  C3  5.0
BOUNDS
 UP BND X  3.0
 FR BND Z
ENDATA
"""


def _read(L, tmp_path, text, name="lp.mps"):
    p = tmp_path / name
    p.write_text(text)
    f = libc.fopen(str(p).encode(), b"r")
    h = L.acdalm_read_mps(f)
    libc.fclose(f)
    return h


def _instance(b, L, h):
    m, n = L.alm_nrhs(h), L.alm_nvars(h)
    mat = L.alm_matrix(h)
    nnz = L.sparse_matrix_nnz(mat)
    coo = [np.ctypeslib.as_array(getattr(L, "sparse_matrix_" + f)(mat), (nnz,)).copy()
           for f in ("rows", "columns", "values")]
    vec = {k: np.ctypeslib.as_array(getattr(L, "alm_" + k)(h), (sz,)).copy()
           for k, sz in (("rhs", m), ("linear", n), ("lower", n), ("upper", n),
                         ("lambda_lower", m), ("lambda_upper", m))}
    return m, n, coo, vec


def test_mps_instance(tmp_path):
    b = binding()
    L = b.lib()
    h = _read(L, tmp_path, LP_MPS)
    assert h, L.acdalm_last_error()
    m, n, (rows, cols, vals), vec = _instance(b, L, h)
    # 4 rows; x, y, z then slacks of C1, C2, C3 (C4 is an equality)
    assert (m, n) == (4, 6)
    dense = np.zeros((m, n))
    dense[rows, cols] = vals
    want = np.array([[1, 1, 0, -1, 0, 0],
                     [1, 3, 0, 0, -1, 0],
                     [0, -1, 1, 0, 0, -1],
                     [1, 0, 1, 0, 0, 0]], float)
    assert (dense == want).all()
    assert (vec["rhs"] == [0, 0, 0, 4]).all()
    assert (vec["linear"] == [-3, -2, 1, 0, 0, 0]).all()
    inf = np.inf
    assert (vec["lower"] == [0, 0, -inf, -inf, -inf, -2]).all()
    assert (vec["upper"] == [3, inf, inf, 4, 6, 3]).all()
    assert (vec["lambda_lower"] == -inf).all() and (vec["lambda_upper"] == inf).all()
    mat = L.alm_matrix(h)
    L.alm_free(h)
    L.sparse_matrix_free(mat)


@pytest.mark.parametrize("sense", ["", "OBJSENSE\n    MAX\n"])
def test_mps_optimum_with_the_oracle(sense, tmp_path, instances, oracle_lib):
    b = binding()
    L = b.lib()
    text = LP_MPS
    if sense:
        # the same LP as a maximisation of the negated objective
        text = text.replace("ROWS", sense + "ROWS", 1)
        text = text.replace("COST  -3.0", "COST  3.0").replace("COST  -2.0", "COST  2.0")
        text = text.replace("Z  COST  1.0", "Z  COST  -1.0")
    h = _read(L, tmp_path, text)
    assert h, L.acdalm_last_error()
    m, n, (rows, cols, vals), vec = _instance(b, L, h)
    lp = instances.LP(m, n, rows.astype(np.uint32), cols.astype(np.uint32), vals,
                      vec["rhs"], vec["linear"], vec["lower"], vec["upper"],
                      vec["lambda_lower"], vec["lambda_upper"], "mps", 0)
    mo = oracle_lib.matrix(lp)
    ho = oracle_lib.alm(mo, lp)
    _, x, lam, diag, _ = oracle_lib.alm_solve(ho, m, n)
    oracle_lib.alm_free(ho)
    oracle_lib.matrix_free(mo)
    assert abs(vec["linear"] @ x - (-10.0)) <= 1e-3
    assert np.allclose(x[:3], [3, 1, 1], atol=1e-3)
    mat = L.alm_matrix(h)
    L.alm_free(h)
    L.sparse_matrix_free(mat)


def test_mps_errors_name_the_line(tmp_path):
    b = binding()
    L = b.lib()
    bad = LP_MPS.replace(" L  C2", " Q  C2")
    assert not _read(L, tmp_path, bad, "bad.mps")
    assert b"line 6" in L.acdalm_last_error()
    assert not _read(L, tmp_path, LP_MPS.replace("ENDATA\n", ""), "noend.mps")
    assert b"ENDATA" in L.acdalm_last_error()
    assert not _read(L, tmp_path, LP_MPS.replace("    RHS  C1  4.0", "    RHS  C9  4.0"),
                     "unknown.mps")
    assert b"unknown row" in L.acdalm_last_error()


def _to_mps(lp):
    """An equality-form LP (bounds finite, multipliers free) as free MPS."""
    lines = ["NAME GEN", "ROWS", " N OBJ"]
    lines += [f" E R{i}" for i in range(lp.nrows)]
    lines.append("COLUMNS")
    order = np.lexsort((lp.rows, lp.cols))
    by_col = {}
    for k in order:
        by_col.setdefault(int(lp.cols[k]), []).append((int(lp.rows[k]), float(lp.vals[k])))
    for j in range(lp.ncols):
        lines.append(f"    C{j} OBJ {float(lp.linear[j])!r}")
        for i, v in by_col.get(j, []):
            lines.append(f"    C{j} R{i} {v!r}")
    lines.append("RHS")
    lines += [f"    RHS R{i} {float(lp.rhs[i])!r}" for i in range(lp.nrows)]
    lines.append("BOUNDS")
    for j in range(lp.ncols):
        lines.append(f" LO BND C{j} {float(lp.lower[j])!r}")
        lines.append(f" UP BND C{j} {float(lp.upper[j])!r}")
    lines.append("ENDATA")
    return "\n".join(lines) + "\n"


def test_equality_lp_round_trips_through_mps(tmp_path, instances):
    """An LP already in equality form comes back unchanged: no slack
    columns, the same triplets and vectors, bit for bit (repr() of a double
    parses back exactly)."""
    b = binding()
    L = b.lib()
    lp = instances.small(seed=12, m=50, n=90, per_col=3)
    h = _read(L, tmp_path, _to_mps(lp), "gen.mps")
    assert h, L.acdalm_last_error()
    m, n, (rows, cols, vals), vec = _instance(b, L, h)
    assert (m, n) == (lp.nrows, lp.ncols)
    got = sorted(zip(rows.tolist(), cols.tolist(), vals.tolist()))
    want = sorted(zip(lp.rows.tolist(), lp.cols.tolist(), lp.vals.tolist()))
    assert got == want
    for k, v in (("rhs", lp.rhs), ("linear", lp.linear), ("lower", lp.lower),
                 ("upper", lp.upper)):
        assert vec[k].tobytes() == np.asarray(v, np.float64).tobytes(), k
    mat = L.alm_matrix(h)
    L.alm_free(h)
    L.sparse_matrix_free(mat)
