"""The oracle (a C restatement of the reference) pinned against the
reference's own outputs: golden fixtures made by running the reference
compiled from its sources (tests/golden/make_golden.py), and, where the
reference sources exist, live comparisons on fresh seeded inputs."""
import hashlib
import os
import tempfile

import numpy as np
import pytest

from golden_io import load_lp, GOLDEN

pytestmark = []


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_layouts_match_reference_fixtures(oracle_lib):
    """Z-order COO, CSR(A), CSR(A'), block arenas, permutations and step
    sizes are byte-identical to what the reference built (spmv.c:27-92,
    approx.c:135-216)."""
    g = np.load(os.path.join(GOLDEN, "layouts.npz"))
    ncase = len({k.split(".")[0] for k in g.files})
    checked = 0
    for idx in range(ncase):
        lp = load_lp(g, f"c{idx}.")
        for perm in (0, 1):
            m = oracle_lib.matrix(lp, bool(perm))
            lay = oracle_lib.layouts(m)
            for key, arrs in lay.items():
                for i, a in enumerate(arrs):
                    want = str(g[f"c{idx}.p{perm}.{key}.{i}"])
                    assert sha(a) == want, (idx, perm, key, i)
                    checked += 1
            a = oracle_lib.approx(m, lp)
            for p in (0, 1):
                d = oracle_lib.internals(a, lp.nrows, lp.ncols, p)
                for k, v in d.items():
                    assert sha(v) == str(g[f"c{idx}.p{perm}.approx{p}.{k}"]), (idx, k)
            oracle_lib.approx_free(a)
            oracle_lib.matrix_free(m)
    assert checked > 100


def test_alm_solve_bit_identical_to_reference(oracle_lib):
    """The full ALM + APPROX solve of the 1,000 x 2,000 workload, including
    the text log, matches the reference bit for bit (alm.c:289-322)."""
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    lp = load_lp(g, "")
    m = oracle_lib.matrix(lp)
    h = oracle_lib.alm(m, lp)
    with tempfile.TemporaryDirectory() as td:
        log = os.path.join(td, "alm.log")
        r, x, lam, diag, used = oracle_lib.alm_solve(h, lp.nrows, lp.ncols, log=log)
        logsha = hashlib.sha256(open(log, "rb").read()).hexdigest()
    oracle_lib.alm_free(h)
    oracle_lib.matrix_free(m)
    assert r == int(g["alm.ret"])
    assert used == int(g["alm.inner"])
    assert x.tobytes() == g["alm.x"].tobytes()
    assert lam.tobytes() == g["alm.lambda"].tobytes()
    assert diag.tobytes() == g["alm.diag"].tobytes()
    assert logsha == str(g["alm.log_sha"])


def test_approx_and_mpg_bit_identical_to_reference(oracle_lib):
    """3,000 APPROX iterations and 50 mpg_solve iterations from x = 0."""
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    lp = load_lp(g, "")
    m = oracle_lib.matrix(lp)
    a = oracle_lib.approx(m, lp)
    r, x, diag = oracle_lib.approx_solve(a, np.zeros(lp.ncols), 3000)
    assert r == int(g["approx.ret"])
    assert x.tobytes() == g["approx.x"].tobytes()
    assert diag.tobytes() == g["approx.diag"].tobytes()
    r, x, diag = oracle_lib.mpg_solve(a, np.zeros(lp.ncols), 50)
    assert r == int(g["mpg.ret"])
    assert x.tobytes() == g["mpg.x"].tobytes()
    assert diag.tobytes() == g["mpg.diag"].tobytes()
    oracle_lib.approx_free(a)
    oracle_lib.matrix_free(m)


def test_solution_is_an_lp_optimum(oracle_lib):
    """The reference solution reaches the 1e-6 relative-KKT bar."""
    import importlib
    inst = importlib.import_module("acd-alm_gb300.instances")
    g = np.load(os.path.join(GOLDEN, "small.npz"))
    lp = load_lp(g, "")
    k = inst.rel_kkt(lp, g["alm.x"], g["alm.lambda"])
    assert k["rel_kkt"] < 1e-6, k


@pytest.mark.parametrize("shape", [(1, 1, 1), (5, 3, 2), (40, 7, 3), (300, 900, 6),
                                   (513, 1027, 5)])
def test_live_against_reference(shape, oracle_lib, ref_lib, instances):
    """Fresh seeded inputs, odd and ragged shapes: every layout and a short
    APPROX run agree with the reference compiled here."""
    m, n, k = shape
    lp = instances.small(seed=7 * m + n, m=m, n=n, per_col=min(k, m))
    for perm in (0, 1):
        mo, mr = oracle_lib.matrix(lp, perm), ref_lib.matrix(lp, perm)
        lo, lr = oracle_lib.layouts(mo), ref_lib.layouts(mr)
        for key in lo:
            for a, b in zip(lo[key], lr[key]):
                assert a.tobytes() == b.tobytes(), key
        x = np.random.default_rng(m).uniform(-1, 1, n)
        assert oracle_lib.multiply(mo, x, 0).tobytes() == ref_lib.multiply(mr, x, 0).tobytes()
        y = np.random.default_rng(n).uniform(-1, 1, m)
        assert oracle_lib.multiply(mo, y, 1).tobytes() == ref_lib.multiply(mr, y, 1).tobytes()
        oracle_lib.matrix_free(mo)
        ref_lib.matrix_free(mr)
    mo, mr = oracle_lib.matrix(lp), ref_lib.matrix(lp)
    ao, ar = oracle_lib.approx(mo, lp), ref_lib.approx(mr, lp)
    ro = oracle_lib.approx_solve(ao, np.ones(n), 400, max_pg=1e-9)
    rr = ref_lib.approx_solve(ar, np.ones(n), 400, max_pg=1e-9)
    assert ro[0] == rr[0]
    assert ro[1].tobytes() == rr[1].tobytes()
    assert ro[2].tobytes() == rr[2].tobytes()


def test_reference_kkt_stop_reproduces_small_fixture(ref_lib, instances):
    """The reference's alm_solve stopped at relative KKT <= 1e-6
    (ref_alm_solve_kkt, one thread) reproduces tests/golden/small_kkt.npz
    bit for bit: the generator behind the KKT-stop fixtures is deterministic."""
    g = np.load(os.path.join(GOLDEN, "small_kkt.npz"))
    lp = instances.small()
    assert lp.sha256() == str(g["instance_sha256"])
    m = ref_lib.matrix(lp)
    h = ref_lib.alm(m, lp)
    r, x, lam, kk, outer, inner = ref_lib.alm_solve_kkt(h, lp.nrows, lp.ncols, 1e-6)
    ref_lib.alm_free(h)
    ref_lib.matrix_free(m)
    assert r == int(g["ret"]) == 0
    assert (outer, inner) == (int(g["outer"]), int(g["inner"]))
    assert kk.tobytes() == g["kkt"].tobytes()
    k = instances.rel_kkt(lp, x, lam)
    assert k["rel_kkt"] <= 1e-6
    assert k["objective"] == float(g["objective"])
