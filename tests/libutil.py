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
