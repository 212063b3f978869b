"""A plain-C caller of the drop-in API (tests/host/alm_driver.c: the
reference's TEST_ALM driver, alm.c:366-395, kept as a caller would keep it
after the switch) compiled with the host C compiler against include/ and
linked with -lacdalm, as INTEGRATION.md describes.

On a machine without a GPU it reports the device failure through the new
negative code and acdalm_last_error() instead of computing; on the GPU it
solves an instance read with alm_read and the objective matches the
oracle's solve of the same LP."""
import os
import re
import shutil
import subprocess
import sys

import pytest

from libutil import ROOT, binding


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    b = binding()
    libdir = os.path.dirname(b.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("ccaller") / "alm_driver")
    subprocess.run([cc, "-std=c11", "-O1", "-Wall", "-Werror",
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "host", "alm_driver.c"),
                    "-L", libdir, "-Wl,-rpath," + libdir, "-lacdalm", "-lm", "-o", exe],
                   check=True)
    return exe


def _instance(instances, tmp_path):
    lp = instances.small(seed=31, m=300, n=600, per_col=5)
    path = str(tmp_path / "lp.txt")
    instances.write_text(lp, path)
    return lp, path


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_c_caller_builds_links_and_reports_a_missing_device(driver, instances, tmp_path):
    if _gpu_present():
        pytest.skip("a GPU is present: test_c_caller_solves_on_the_gpu covers it")
    lp, path = _instance(instances, tmp_path)
    r = subprocess.run([driver, path], capture_output=True, text=True)
    assert r.returncode == 2, (r.returncode, r.stdout, r.stderr)
    assert re.search(r"alm_solve: -6: ", r.stderr), r.stderr   # ACDALM_ENODEV


@pytest.mark.gpu
def test_c_caller_solves_on_the_gpu(driver, instances, tmp_path):
    lp, path = _instance(instances, tmp_path)
    r = subprocess.run([driver, path], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    m = re.search(r"ret (\d) objective (\S+) max_violation (\S+)", r.stdout)
    assert m, r.stdout
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if not oracle.available("oracle"):
        oracle.build(ref=False)
    o = oracle.Lib("oracle")
    mo = o.matrix(lp)
    ho = o.alm(mo, lp)
    ro, xo, lo, do, _ = o.alm_solve(ho, lp.nrows, lp.ncols)
    o.alm_free(ho)
    o.matrix_free(mo)
    assert int(m.group(1)) == ro
    obj = float(m.group(2))
    ref = float(lp.linear @ xo)
    assert abs(obj - ref) <= 1e-6 * (abs(ref) + 1), (obj, ref)
