"""Loader for the golden fixtures written by tests/golden/make_golden.py."""

import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

_cache = None


def load():
    global _cache
    if _cache is None:
        with open(os.path.join(HERE, "golden.json")) as f:
            index = json.load(f)
        arrays = dict(np.load(os.path.join(HERE, "golden.npz")))
        cases = []
        for c in index["cases"]:
            case = dict(c)
            case["inputs"] = {k: arrays[v] for k, v in c["inputs"].items()}
            case["outputs"] = {k: arrays[v] for k, v in c["outputs"].items()}
            cases.append(case)
        _cache = cases
    return _cache


def cases(kind=None):
    return [c for c in load() if kind is None or c["kind"] == kind]


def unpack_shapelets(case):
    packed = case["inputs"]["shapelets"]
    lens = case["inputs"]["lengths"]
    out, off = [], 0
    for n in lens:
        out.append(packed[off:off + int(n)])
        off += int(n)
    return out
