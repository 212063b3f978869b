"""The LP server's admission rule (acd-alm_gb300/csrc/admission.h), compiled
on its own with the host compiler and checked on small scenarios: the
order (one-CTA requests by arrival, then clusters by most nonzeros), SM and
memory accounting, backfilling, and the wait limit after which a request
blocks the ones behind it."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "acd-alm_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path_factory.mktemp("admission") / "admission_driver")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", CSRC,
                    os.path.join(HERE, "host", "admission_driver.cpp"), "-o", exe],
                   check=True)

    def run(lines):
        out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True,
                             text=True, check=True).stdout.split("\n")
        return out[:len(lines)]
    return run


def test_order_one_cta_first_then_clusters_by_nonzeros(driver):
    # id nnz team
    got = driver(["order 0 2000000 16  1 50000 1  2 700000 8  3 90000 1  4 2000000 16  5 300000 4"])
    assert got == ["1 3 0 4 2 5"]


def test_pick_takes_the_first_request_that_fits(driver):
    # sms busy budget in_use running backfill | id nnz team footprint waited
    got = driver([
        "pick 152 150 1000 0 1 10  0 2000000 16 100 0  1 50000 1 10 0",
        "pick 152 140 1000 0 1 10  0 2000000 16 100 0  1 50000 1 10 0",
        "pick 152 130 1000 0 1 10  0 2000000 16 100 0  1 50000 1 10 0",
    ])
    assert got == ["1", "1", "0"]


def test_pick_respects_the_memory_budget(driver):
    got = driver([
        "pick 152 0 1000 950 1 10  0 50000 1 100 0  1 40000 1 40 0",
        "pick 152 0 1000 990 1 10  0 50000 1 100 0  1 40000 1 40 0",
    ])
    assert got == ["1", "-1"]


def test_a_request_that_waited_too_long_blocks_the_ones_behind_it(driver):
    got = driver([
        "pick 152 140 1000 0 1 10  0 2000000 16 100 9.5  1 50000 1 10 0",
        "pick 152 140 1000 0 1 10  0 2000000 16 100 10.5  1 50000 1 10 0",
    ])
    assert got == ["1", "-1"]


def test_with_nothing_running_the_first_request_goes_whatever_its_size(driver):
    got = driver([
        "pick 16 0 1000 0 0 10  0 9000000 16 5000 0  1 50000 1 10 0",
        "pick 152 0 1000 0 1 10",
    ])
    assert got == ["0", "-1"]
