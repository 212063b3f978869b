"""Binary instances (acdalm_write_binary / acdalm_read_binary): the same
content as alm_read's text format (alm.c:330-364), read back into an
identical instance -- the same matrix triplets (in the matrix's own COO
order) and the same vectors; truncated or foreign streams are refused.
Host-only: no GPU needed."""
import ctypes

import numpy as np

from libutil import binding

libc = ctypes.CDLL(None)
libc.fopen.restype = ctypes.c_void_p
libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
libc.fclose.argtypes = [ctypes.c_void_p]


def _vec(L, name, h, n):
    return np.ctypeslib.as_array(getattr(L, "alm_" + name)(h), (max(n, 1),))[:n].copy()


def _coo(L, mat):
    n = L.sparse_matrix_nnz(mat)
    return [np.ctypeslib.as_array(getattr(L, "sparse_matrix_" + f)(mat), (max(n, 1),))[:n].copy()
            for f in ("rows", "columns", "values")]


def _lp(instances):
    lp = instances.small(seed=9, m=60, n=150, per_col=3)
    rng = np.random.default_rng(4)
    lp.lambda_lower = rng.uniform(-5, 0, lp.nrows)
    lp.lambda_upper = rng.uniform(0, 5, lp.nrows)
    return lp


def test_round_trip(instances, tmp_path):
    b = binding()
    L = b.lib()
    lp = _lp(instances)
    m = b.Matrix(lp)
    a = b.Alm(m, lp)
    path = str(tmp_path / "lp.bin").encode()
    f = libc.fopen(path, b"wb")
    assert L.acdalm_write_binary(a.h, f) == 0
    libc.fclose(f)
    f = libc.fopen(path, b"rb")
    h = L.acdalm_read_binary(f)
    libc.fclose(f)
    assert h
    assert L.alm_nrhs(h) == lp.nrows and L.alm_nvars(h) == lp.ncols
    for name, n in (("rhs", lp.nrows), ("linear", lp.ncols), ("lower", lp.ncols),
                    ("upper", lp.ncols), ("lambda_lower", lp.nrows),
                    ("lambda_upper", lp.nrows)):
        assert _vec(L, name, h, n).tobytes() == _vec(L, name, a.h, n).tobytes(), name
    mat = L.alm_matrix(h)
    for got, want in zip(_coo(L, mat), _coo(L, m.h)):
        assert got.tobytes() == want.tobytes()
    L.alm_free(h)
    L.sparse_matrix_free(mat)
    a.free()
    m.free()


def test_truncated_and_foreign_streams_are_refused(instances, tmp_path):
    b = binding()
    L = b.lib()
    lp = _lp(instances)
    m = b.Matrix(lp)
    a = b.Alm(m, lp)
    full = tmp_path / "lp.bin"
    f = libc.fopen(str(full).encode(), b"wb")
    assert L.acdalm_write_binary(a.h, f) == 0
    libc.fclose(f)
    data = full.read_bytes()
    for name, content in (("short.bin", data[:-8]), ("text.bin", b"1 1 1\n0 0 1\n" + data)):
        p = tmp_path / name
        p.write_bytes(content)
        f = libc.fopen(str(p).encode(), b"rb")
        assert not L.acdalm_read_binary(f), name
        libc.fclose(f)
        assert b"acdalm_read_binary" in L.acdalm_last_error()
    a.free()
    m.free()
