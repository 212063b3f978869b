"""Loading the golden fixtures written by tests/golden/make_golden.py."""
import importlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_lp(g, prefix: str):
    inst = importlib.import_module("acd-alm_gb300.instances")
    shape = g[prefix + "shape"]
    return inst.LP(nrows=int(shape[0]), ncols=int(shape[1]),
                   rows=g[prefix + "rows"], cols=g[prefix + "cols"],
                   vals=g[prefix + "vals"], rhs=g[prefix + "rhs"],
                   linear=g[prefix + "linear"], lower=g[prefix + "lower"],
                   upper=g[prefix + "upper"],
                   lambda_lower=g[prefix + "lambda_lower"],
                   lambda_upper=g[prefix + "lambda_upper"])
