"""Helpers shared by the library tests: loading libacdalm and its Python
binding, and skipping GPU tests cleanly."""
import importlib
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def binding():
    """The package's ctypes binding (acd-alm_gb300/lib.py), building the
    library first if it is missing."""
    b = importlib.import_module("acd-alm_gb300.lib")
    if not os.path.exists(b.LIB_PATH):
        importlib.import_module("acd-alm_gb300.build_lib").build()
    return b


def header_functions():
    """Every function declared in include/*.h."""
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            pre = text[:m.start()].rstrip()
            if name in ("if", "sizeof", "return", "defined") or pre.endswith("(*"):
                continue
            # a declaration: preceded by a type, not inside typedef (*fn)
            line = text[text.rfind("\n", 0, m.start()) + 1:m.start()]
            if line.strip().startswith("#") or "typedef" in line:
                continue
            names.add(name)
    return names


def ragged_lp(instances, seed, m=300, n=900):
    """An LP whose rows have lengths 0..700 (every lane count and both slice
    kinds of the SELL layout), with some stored zeros; columns of lengths
    0..hundreds.  Bounds 0 <= x <= 1, b = A x0 for a feasible x0."""
    import numpy as np
    rng = np.random.default_rng(seed)
    lens = np.concatenate([np.zeros(5, int), rng.integers(1, 17, 150),
                           rng.integers(17, 65, 80), rng.integers(65, 257, 50),
                           rng.integers(257, 700, 15)])[:m]
    lens = np.concatenate([lens, rng.integers(1, 9, m - lens.size)]).astype(int)
    rows, cols = [], []
    for r, k in enumerate(lens):
        k = min(int(k), n)
        rows.append(np.full(k, r))
        cols.append(np.sort(rng.choice(n, k, replace=False)))
    rows = np.concatenate(rows).astype(np.uint32)
    cols = np.concatenate(cols).astype(np.uint32)
    vals = rng.uniform(-1, 1, rows.size)
    vals[::13] = 0.0
    x0 = rng.uniform(0, 1, n)
    lp = instances.LP(m, n, rows, cols, vals, np.zeros(m), rng.uniform(-1, 1, n),
                      np.zeros(n), np.ones(n), np.full(m, -np.inf), np.full(m, np.inf),
                      "ragged", seed)
    lp.rhs = lp.matvec(x0)
    return lp
