"""Comparison helpers shared by the tests."""
import numpy as np


def same_bits(a, b):
    """Bit-identical float arrays, except that any NaN matches any NaN (the
    sign and payload of a NaN produced from 0/0 are not specified by IEEE)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind != "f":
        return np.array_equal(a, b)
    an, bn = np.isnan(a), np.isnan(b)
    if not np.array_equal(an, bn):
        return False
    iv = np.uint32 if a.dtype == np.float32 else np.uint64
    return np.array_equal(a.view(iv)[~an], b.view(iv)[~bn])


def first_diff(a, b):
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    n = min(a.size, b.size)
    if a.dtype.kind == "f":
        iv = np.uint32 if a.dtype == np.float32 else np.uint64
        d = np.nonzero((a[:n].view(iv) != b[:n].view(iv)) & ~(np.isnan(a[:n]) & np.isnan(b[:n])))[0]
    else:
        d = np.nonzero(a[:n] != b[:n])[0]
    if d.size == 0:
        return None if a.size == b.size else ("size", a.size, b.size)
    i = int(d[0])
    return (i, a[i], b[i], int(d.size))


# ------------------------------------------------------------------ golden fixtures

import json as _json
import os as _os

GOLDEN_DIR = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "golden")
_golden = None


def golden():
    """(manifest list, npz arrays) of tests/golden (made by make_golden.py)."""
    global _golden
    if _golden is None:
        man = _json.load(open(_os.path.join(GOLDEN_DIR, "cases.json")))
        arr = np.load(_os.path.join(GOLDEN_DIR, "golden.npz"))
        _golden = (man, arr)
    return _golden


def golden_inputs(entry, arr):
    v = arr[f"{entry['case']}__input"]
    rect = arr[f"{entry['case']}__rect"] if entry["rect"] else None
    return v, rect


def golden_outputs(entry, arr):
    k = entry["key"]
    return {f: arr[f"{k}__{f}"] for f in ("coords", "normals", "connections", "colors")}
