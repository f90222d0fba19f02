"""Loading the golden fixtures of tests/golden (made by tests/golden/make_golden.py
from the reference's own programs)."""
import json
import os

import numpy as np

import su

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d)))
ATTRS = {"cmp": ["c", "coher", "stack"], "crs": ["a", "b", "c", "coher", "stack"]}
SHIPPED = {"cmp": "f32", "crs": "f64"}


def load(name):
    d = os.path.join(GOLDEN, name)
    with open(os.path.join(d, "args.json")) as f:
        meta = json.load(f)
    h, s = su.read_su(os.path.join(d, "in.su"))
    return meta, h, s, os.path.join(d, "in.su")


def binary_dir(method, prec):
    shipped = SHIPPED[method]
    tag = "" if prec == shipped else "-" + {"f32": "fp32", "f64": "fp64"}[prec]
    return f"{method}-omp2{tag}"


def ref_outputs(name, method, prec):
    d = os.path.join(GOLDEN, name, binary_dir(method, prec))
    return {k: su.read_su(os.path.join(d, f"{method}.{k}.su")) for k in ATTRS[method]}


def ref_file(name, method, prec, attr):
    return os.path.join(GOLDEN, name, binary_dir(method, prec), f"{method}.{attr}.su")


def rows_by_cdp(cdp_ids, headers):
    """Row index in cdp_ids order of each output trace (outputs are keyed by cdp)."""
    pos = {int(c): i for i, c in enumerate(cdp_ids)}
    return np.array([pos[int(c)] for c in headers["cdp"]])
