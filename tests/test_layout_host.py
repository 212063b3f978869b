"""Host layouts built by the library (no GPU needed) are byte-identical to
the reference's: the golden fixtures made from the reference itself, and
live comparisons with the oracle on fresh inputs (spmv.c:27-92,
permutation.c:63-125, spmv_csr.c:27-80, spmv_block.c:58-149,
spmv.swizzle.inc:14-52)."""
import hashlib
import os

import numpy as np
import pytest

from golden_io import GOLDEN, load_lp
from libutil import binding, ragged_lp


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_layouts_match_reference_fixtures():
    b = binding()
    g = np.load(os.path.join(GOLDEN, "layouts.npz"))
    ncase = len({k.split(".")[0] for k in g.files})
    for idx in range(ncase):
        lp = load_lp(g, f"c{idx}.")
        for perm in (0, 1):
            m = b.Matrix(lp, permute=bool(perm))
            for key, arrs in m.layouts().items():
                for i, a in enumerate(arrs):
                    assert sha(a) == str(g[f"c{idx}.p{perm}.{key}.{i}"]), (idx, perm, key, i)
            m.free()


def test_permuted_shadow_matches_reference_fixture():
    """approx_make's permuted copy (approx.c:84-88) has the reference's
    layouts (its step sizes are checked on the GPU)."""
    b = binding()
    g = np.load(os.path.join(GOLDEN, "layouts.npz"))
    lp = load_lp(g, "c3.")
    m = b.Matrix(lp)
    a = b.Approx(m, lp)
    pm = a.permuted_matrix()
    for key, arrs in pm.layouts().items():
        for i, arr in enumerate(arrs):
            assert sha(arr) == str(g[f"c3.p1.{key}.{i}"]), (key, i)
    a.free()
    m.free()


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 9, 2), (31, 64, 3), (257, 513, 7),
                                   (1000, 700, 1)])
def test_layouts_match_oracle_live(shape, oracle_lib, instances):
    b = binding()
    m_, n_, k = shape
    lp = instances.small(seed=m_ + 3 * n_, m=m_, n=n_, per_col=min(k, m_))
    for perm in (0, 1):
        mine = b.Matrix(lp, permute=bool(perm))
        mo = oracle_lib.matrix(lp, perm)
        lo = oracle_lib.layouts(mo)
        for key, arrs in mine.layouts().items():
            for a, o in zip(arrs, lo[key]):
                assert a.tobytes() == o.tobytes(), key
        oracle_lib.matrix_free(mo)
        mine.free()


def test_zero_values_take_ring_columns(instances):
    """A stored 0.0 is treated as padding by the block builder (its column
    comes from the ring, spmv_block.c:152-160), like the reference."""
    b = binding()
    lp = instances.small(seed=5, m=40, n=60, per_col=4)
    lp.vals[::7] = 0.0
    import oracle as O
    o = O.Lib("oracle")
    mo = o.matrix(lp, 0)
    mine = b.Matrix(lp)
    assert mine.layouts()["block0"][1].tobytes() == o.layouts(mo)["block0"][1].tobytes()
    o.matrix_free(mo)
    mine.free()


def test_permute_vectors(instances):
    """sparse_matrix_{row,col}_permute: forward gathers with idx, inverse
    with ridx; a wrong length returns 1 (permutation.c:136-148)."""
    b = binding()
    lp = instances.small(seed=8, m=50, n=80, per_col=3)
    m = b.Matrix(lp, permute=True)
    lay = m.layouts()
    idx, ridx = lay["cperm"]
    src = np.arange(lp.ncols, dtype=np.float64)
    dst = np.zeros(lp.ncols)
    L = b.lib()
    assert L.sparse_matrix_col_permute(m.h, dst, lp.ncols, src, 1) == 0
    assert (dst == src[idx]).all()
    back = np.zeros(lp.ncols)
    assert L.sparse_matrix_col_permute(m.h, back, lp.ncols, dst, -1) == 0
    assert (back == src).all()
    assert L.sparse_matrix_col_permute(m.h, back, lp.ncols - 1, dst, -1) == 1
    m.free()


def _decode_sell(s, nrows):
    """Row d of the SELL layout as (columns, values), padding included, and
    the number of vector slices."""
    out = {}
    ptr = s["ptr"]
    nvec = 0
    for sl in range(len(s["row0"])):
        L = 1 << int(ptr[sl] & 7)
        V = 4 if ptr[sl] & 8 else 1
        nvec += V == 4
        base = int(ptr[sl]) & ~31
        span = (int(ptr[sl + 1]) & ~31) - base
        assert span % (32 * V) == 0
        steps = span // (32 * V)
        for r in range(32 // L):
            d = int(s["row0"][sl]) + r
            k = np.arange(steps * V * L)
            at = base + 32 * V * (k // (V * L)) + V * (r * L + (k // V) % L) + k % V
            out[d] = (s["col"][at], s["val"][at])
    assert sorted(out) == list(range(len(out))) and len(out) >= nrows
    return out, nvec


@pytest.mark.parametrize("mode", ["0", "1", "auto"])
@pytest.mark.parametrize("transpose", [False, True])
def test_sell_layout_holds_every_row_in_order(instances, transpose, mode, monkeypatch):
    """The SELL layout (scalar slices: 1 entry per lane per step; vector
    slices: 4) holds each row's entries in CSR order followed by
    zero-valued padding whose columns are in range; rows are in decreasing
    length.  ACDALM_SELL_VEC picks scalar (0), vector (1) or per-slice
    (auto) slices."""
    b = binding()
    lp = ragged_lp(instances, 4)
    m = b.Matrix(lp)
    monkeypatch.setenv("ACDALM_SELL_VEC", mode)
    s = m.sell(transpose)
    ri, cc, vv = m.layouts()[f"csr{int(transpose)}"]
    nrows, ncols = (lp.ncols, lp.nrows) if transpose else (lp.nrows, lp.ncols)
    rows, nvec = _decode_sell(s, nrows)
    nslices = len(s["row0"])
    assert nvec == {"0": 0, "1": nslices}.get(mode, nvec)
    if mode == "auto":
        assert 0 < nvec < nslices
    assert sorted(s["row_of_d"]) == list(range(nrows))
    lens = np.diff(ri.astype(np.int64))
    assert (np.diff(lens[s["row_of_d"]]) <= 0).all()
    for d in range(nrows):
        r = s["row_of_d"][d]
        k = lens[r]
        c, v = rows[d]
        assert (c[:k] == cc[ri[r]:ri[r + 1]]).all() and (v[:k] == vv[ri[r]:ri[r + 1]]).all()
        assert (v[k:] == 0).all() and (c >= 0).all() and (c < ncols).all()
    for d in range(nrows, len(rows)):
        c, v = rows[d]
        assert (v == 0).all() and (c >= 0).all() and (c < ncols).all()
    m.free()
