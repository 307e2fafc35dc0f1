"""Access to the golden fixtures in tests/golden (made by make_golden.py)."""
import json
import os

import numpy as np

from tskit_gb300.tables import Tables

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


def load(name):
    data = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    tables = Tables.from_npz(data, prefix="tables/")
    return tables, data


def resolve(kwargs, data):
    kw = dict(kwargs)
    for k, v in kw.items():
        if isinstance(v, str) and v.startswith("@"):
            kw[k] = data[v[1:]]
    if "time_windows" in kw:
        kw["time_windows"] = np.array(kw["time_windows"], dtype=np.float64)
    return kw


def all_cases():
    out = []
    for name, cases in manifest().items():
        for c in cases:
            if "key" in c:
                out.append((name, c))
    return out
