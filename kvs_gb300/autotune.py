"""Launch-shape autotuning of the streaming kernels (kvsmc_autotune and the
tuning table of include/kvsmc.h).

A shape is four integers: ``rows`` (cell rows per warp task, 1 or 2),
``tasks_per_sm`` (warp tasks per SM a launch is cut into), ``ctas_per_sm``
(resident CTAs per SM of the persistent launches) and ``scan_threads`` (the
unit-scan tile).  0 in any field means the built-in rule.  A table holds one
shape per (value type, size class); every streaming batch, plan and server
round of a context follows the table installed on it.  Shapes never change
results, only speed.

    table = autotune(ctx)            # times candidates, installs the table
    save("tuning.json", table)
    install(other_ctx, load("tuning.json"))

The reference runs one CPU loop per call and has nothing to tune.
"""
import ctypes as C
import json

import numpy as np

from . import _abi

FIELDS = ("rows", "tasks_per_sm", "ctas_per_sm", "scan_threads")
FORMAT = "kvsmc-tuning-1"


def size_class(nx, ny, nz):
    """Size class (0..4) of a volume with nx x ny x nz nodes."""
    return int(_abi.load().kvsmc_size_class(int(nx), int(ny), int(nz)))


def _dtype_name(code):
    return np.dtype(_abi.DTYPES[code]).name


def _to_entries(table):
    arr = (_abi.TuneEntry * max(1, len(table)))()
    for i, row in enumerate(table):
        e = arr[i]
        e.dtype = _abi.dtype_code(row["dtype"])
        e.size_class = int(row["size_class"])
        for f in FIELDS:
            setattr(e.choice, f, int(row.get(f, 0)))
        e.tuned_ms = float(row.get("tuned_ms", 0.0))
        e.default_ms = float(row.get("default_ms", 0.0))
    return arr


def _from_entries(arr, n):
    out = []
    for i in range(n):
        e = arr[i]
        row = {"dtype": _dtype_name(e.dtype), "size_class": int(e.size_class)}
        for f in FIELDS:
            row[f] = int(getattr(e.choice, f))
        row["tuned_ms"] = float(e.tuned_ms)
        row["default_ms"] = float(e.default_ms)
        out.append(row)
    return out


def resolve(table, dtype, nx, ny, nz):
    """The shape a streaming batch uses for a volume under `table` (list of
    rows as returned by autotune / load; empty: the built-in rules)."""
    lib = _abi.load()
    arr = _to_entries(table)
    c = _abi.TuneChoice()
    st = lib.kvsmc_tune_resolve(arr if table else None, len(table), _abi.dtype_code(dtype),
                                int(nx), int(ny), int(nz), C.byref(c))
    if st:
        raise _abi.KvsmcError(st, "tune_resolve: " + _abi.status_string(st))
    return {f: int(getattr(c, f)) for f in FIELDS}


def install(ctx, table):
    """Install a table on a context (empty list: back to the built-in rules)."""
    arr = _to_entries(table)
    ctx.check(ctx.lib.kvsmc_tuning_set(ctx.handle, arr if table else None, len(table)), "tuning_set")


def installed(ctx):
    """The table installed on a context."""
    n = ctx.lib.kvsmc_tuning_get(ctx.handle, None, 0)
    arr = (_abi.TuneEntry * max(1, n))()
    n = ctx.lib.kvsmc_tuning_get(ctx.handle, arr, n)
    return _from_entries(arr, n)


def force(ctx, shape=None):
    """Use one shape for every volume of the context (None: the table)."""
    if shape is None:
        ctx.check(ctx.lib.kvsmc_tuning_force(ctx.handle, None), "tuning_force")
        return
    c = _abi.TuneChoice(*(int(shape.get(f, 0)) for f in FIELDS))
    ctx.check(ctx.lib.kvsmc_tuning_force(ctx.handle, C.byref(c)), "tuning_force")


def autotune(ctx, dtypes=None, max_class=_abi.SIZE_CLASSES - 1, isovalues=4, reps=3, seed=1):
    """Run the autotuner on the context's device; installs and returns the
    table (one row per (dtype, size class), with the measured times)."""
    cfg = _abi.AutotuneConfig()
    keep = None
    if dtypes is not None:
        codes = [_abi.dtype_code(d) for d in dtypes]
        keep = (C.c_int32 * len(codes))(*codes)
        cfg.dtypes = C.cast(keep, C.POINTER(C.c_int32))
        cfg.ndtypes = len(codes)
    cfg.max_class = int(max_class)
    cfg.isovalues = int(isovalues)
    cfg.reps = int(reps)
    cfg.seed = int(seed)
    cap = 5 * _abi.SIZE_CLASSES
    arr = (_abi.TuneEntry * cap)()
    n = C.c_int32(0)
    ctx.check(ctx.lib.kvsmc_autotune(ctx.handle, C.byref(cfg), arr, cap, C.byref(n)), "autotune")
    del keep
    return _from_entries(arr, n.value)


def save(path, table):
    with open(path, "w") as f:
        json.dump({"format": FORMAT, "entries": table}, f, indent=1)


def load(path):
    with open(path) as f:
        doc = json.load(f)
    if doc.get("format") != FORMAT:
        raise ValueError(f"{path}: not a {FORMAT} table")
    table = doc["entries"]
    resolve(table, np.float32, 2, 2, 2)   # validates every row
    return table
