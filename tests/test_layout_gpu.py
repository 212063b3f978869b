"""The reference's layouts built on the GPU (acdalm_layout_device): the
nonzero-count permutations (spmv/permutation.c:63-125) and the CSR of A and
A' (spmv/spmv_csr.c:27-80), byte for byte the reference's -- against the
golden fixtures made by running the reference (tests/golden/layouts.npz)
and against the host builders on ragged and random matrices."""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from golden_io import GOLDEN, load_lp
from libutil import binding, ragged_lp

pytestmark = pytest.mark.gpu

_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _entry(L):
    f = L.acdalm_layout_device
    f.restype = ctypes.c_int
    f.argtypes = [_sz, _sz, _sz] + [_vp] * 3 + [ctypes.c_int] + [_vp] * 8 + [_vp]
    return f


def device_layouts(lp, permute):
    """The layouts as acdalm_layout_device builds them, as numpy arrays with
    the keys of Matrix.layouts()."""
    import torch
    L = binding().lib()
    f = _entry(L)
    dev = "cuda"
    as_t = lambda a, dt: torch.tensor(np.ascontiguousarray(a).view(dt), device=dev)
    rows = as_t(lp.rows.astype(np.uint32), np.int32)
    cols = as_t(lp.cols.astype(np.uint32), np.int32)
    vals = torch.tensor(np.ascontiguousarray(lp.vals, np.float64), device=dev)
    m, n, nnz = lp.nrows, lp.ncols, lp.nnz
    ri = torch.zeros(max(m, 1), dtype=torch.int32, device=dev)
    ci = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    ptr = torch.zeros(m + 1, dtype=torch.int32, device=dev)
    col = torch.zeros(max(nnz, 1), dtype=torch.int32, device=dev)
    val = torch.zeros(max(nnz, 1), dtype=torch.float64, device=dev)
    ptr_t = torch.zeros(n + 1, dtype=torch.int32, device=dev)
    col_t = torch.zeros(max(nnz, 1), dtype=torch.int32, device=dev)
    val_t = torch.zeros(max(nnz, 1), dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    r = f(m, n, nnz, rows.data_ptr(), cols.data_ptr(), vals.data_ptr(), int(permute),
          ri.data_ptr(), ci.data_ptr(), ptr.data_ptr(), col.data_ptr(), val.data_ptr(),
          ptr_t.data_ptr(), col_t.data_ptr(), val_t.data_ptr(), s)
    assert r == 0, L.acdalm_last_error()
    u = lambda t, k: t.cpu().numpy().view(np.uint32)[:k]
    return {"rperm.0": u(ri, m), "cperm.0": u(ci, n),
            "csr0.0": u(ptr, m + 1), "csr0.1": u(col, nnz), "csr0.2": val.cpu().numpy()[:nnz],
            "csr1.0": u(ptr_t, n + 1), "csr1.1": u(col_t, nnz),
            "csr1.2": val_t.cpu().numpy()[:nnz]}


def test_device_layouts_match_reference_fixtures():
    g = np.load(os.path.join(GOLDEN, "layouts.npz"))
    ncase = len({k.split(".")[0] for k in g.files})
    for idx in range(ncase):
        lp = load_lp(g, f"c{idx}.")
        for perm in (0, 1):
            for key, a in device_layouts(lp, perm).items():
                assert sha(a) == str(g[f"c{idx}.p{perm}.{key}"]), (idx, perm, key)


@pytest.mark.parametrize("permute", [0, 1])
def test_device_layouts_match_host_builders(permute, instances):
    b = binding()
    cases = [ragged_lp(instances, 31), instances.small(seed=32, m=3000, n=7000, per_col=7),
             instances.covering(m=2000, n=6000)]
    # rows and columns without entries
    e = instances.small(seed=33, m=300, n=500, per_col=2)
    keep = (e.cols % 5 != 0) & (e.rows % 7 != 0)
    e.rows, e.cols, e.vals = e.rows[keep], e.cols[keep], e.vals[keep]
    cases.append(e)
    for lp in cases:
        m = b.Matrix(lp, permute=bool(permute))
        host = m.layouts()
        dev = device_layouts(lp, permute)
        for key, a in dev.items():
            name, i = key.split(".")
            assert a.tobytes() == host[name][int(i)].tobytes(), (lp.name, key)
        m.free()


def test_device_layouts_of_an_empty_matrix(instances):
    lp = instances.small(seed=34, m=10, n=20, per_col=1)
    lp.rows, lp.cols, lp.vals = lp.rows[:0], lp.cols[:0], lp.vals[:0]
    d = device_layouts(lp, 1)
    assert (d["csr0.0"] == 0).all() and (d["csr1.0"] == 0).all()
    assert sorted(d["rperm.0"]) == list(range(10))


def test_out_of_range_triplets_are_refused(instances):
    import torch
    L = binding().lib()
    f = _entry(L)
    lp = instances.small(seed=35, m=50, n=80, per_col=3)
    rows = lp.rows.astype(np.uint32).copy()
    rows[5] = lp.nrows  # one past the last row
    dt = lambda a: torch.tensor(a.view(np.int32), device="cuda")
    r_, c_ = dt(rows), dt(lp.cols.astype(np.uint32))
    v_ = torch.tensor(lp.vals, device="cuda")
    out = [torch.zeros(max(k, 1), dtype=torch.int32, device="cuda")
           for k in (lp.nrows, lp.ncols, lp.nrows + 1, lp.nnz)]
    val = torch.zeros(lp.nnz, dtype=torch.float64, device="cuda")
    out_t = [torch.zeros(max(k, 1), dtype=torch.int32, device="cuda")
             for k in (lp.ncols + 1, lp.nnz)]
    val_t = torch.zeros(lp.nnz, dtype=torch.float64, device="cuda")
    r = f(lp.nrows, lp.ncols, lp.nnz, r_.data_ptr(), c_.data_ptr(), v_.data_ptr(), 1,
          out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(),
          val.data_ptr(), out_t[0].data_ptr(), out_t[1].data_ptr(), val_t.data_ptr(), None)
    assert r == -4 and b"out of range" in L.acdalm_last_error()
