"""Launch shapes of the streaming kernels and the autotuner.

A shape (rows per warp task, warp tasks per SM, CTAs per SM, unit-scan tile)
changes how the work is cut, never the result: under every shape a batch must
give the same bits as under the built-in rules (which test_stream_gpu.py pins
to the gather kernels and the oracle), in single batches, in replayed plans
and after the autotuner installs its table.
"""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import autotune as T
from kvs_gb300 import synthetic as S

from .test_plan_gpu import _requests
from .test_stream_gpu import compare, extract_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = [
    {"rows": 1, "tasks_per_sm": 24},
    {"rows": 2, "tasks_per_sm": 384, "ctas_per_sm": 1, "scan_threads": 64},
    {"rows": 1, "tasks_per_sm": 4096, "scan_threads": 128},
    {"rows": 2, "tasks_per_sm": 1},
    {"ctas_per_sm": 2, "scan_threads": 256},
]


def _sparse():
    v = np.zeros((60, 40, 290), np.float32)
    v[30:42, 10:20, 150:180] = S.to_numpy(S.gaussian_blobs((12, 10, 30), seed=41))
    return v


def _volumes(ctx):
    rng = np.random.default_rng(40)
    fields = [
        (S.to_numpy(S.fbm((33, 45, 70), seed=42)), [0.3, 0.5, 0.62]),
        (S.to_numpy(S.ellipsoid_phantom((21, 30, 300), np.uint8, seed=43)), [60.5, 140.0]),   # two 256-cell segments
        (S.to_numpy(S.ellipsoid_phantom((25, 26, 90), np.uint16, seed=44)), [20000.5]),
        (rng.integers(-3000, 3000, (12, 13, 140)).astype(np.int16), [0.5, 700.0]),
        (rng.integers(-100, 100, (9, 10, 11)).astype(np.int8), [3.5]),
        (_sparse(), [0.5, 0.2]),                                                             # brick skipping
    ]
    vols, params = [], []
    for v, isos in fields:
        dv = _abi.DeviceVolume.upload(ctx, v)
        for iso in isos:
            vols.append(dv)
            params.append(_abi.make_params(iso, 0))
    return vols, params


@pytest.fixture
def clean_tuning(kvsmc_ctx):
    T.force(kvsmc_ctx, None)
    T.install(kvsmc_ctx, [])
    yield kvsmc_ctx
    T.force(kvsmc_ctx, None)
    T.install(kvsmc_ctx, [])


def test_every_shape_gives_the_same_bits(clean_tuning):
    ctx = clean_tuning
    vols, params = _volumes(ctx)
    ref = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    for shape in SHAPES:
        T.force(ctx, shape)
        got = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
        for i in range(len(params)):
            assert got[i]["status"] == 0
            compare(got[i], ref[i], f"{shape} request {i}")
        # each volume alone, too (one launch kind, different z-chunking)
        for i in (0, 3, 8):
            one = extract_batch(ctx, [vols[i]], [params[i]], _abi.PATH_AUTO)
            compare(one[0], ref[i], f"{shape} alone {i}")


def test_installed_table_is_followed(clean_tuning):
    """A table row for one (dtype, class) changes only the volumes it names;
    results stay identical."""
    ctx = clean_tuning
    vols, params = _volumes(ctx)
    ref = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    table = [{"dtype": d, "size_class": c, "rows": 2, "tasks_per_sm": 7, "ctas_per_sm": 1, "scan_threads": 64}
             for d in ("float32", "uint8", "uint16", "int16", "int8") for c in range(_abi.SIZE_CLASSES)]
    T.install(ctx, table)
    assert T.installed(ctx)[0]["tasks_per_sm"] == 7
    got = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    for i in range(len(params)):
        compare(got[i], ref[i], f"table request {i}")


def test_plan_under_forced_shape(clean_tuning):
    ctx = clean_tuning
    vols, params = _volumes(ctx)
    ref = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    T.force(ctx, SHAPES[1])
    reqs, bufs = _requests(vols, params)
    plan = _abi.Plan(ctx, reqs)
    T.force(ctx, None)    # the plan keeps the shape it was made with
    for _ in range(2):
        plan.launch()
        plan.wait()
        for i in range(len(params)):
            n = reqs[i].sizes.ntriangles
            got = dict(coords=bufs[i][0][:9 * n].cpu().numpy(), normals=bufs[i][1][:3 * n].cpu().numpy(), ntri=n)
            compare(got, ref[i], f"plan request {i}")
    plan.close()


def test_bad_shapes_are_refused(clean_tuning):
    ctx = clean_tuning
    for bad in ({"rows": 3}, {"scan_threads": 96}, {"ctas_per_sm": -1}):
        with pytest.raises(_abi.KvsmcError):
            T.force(ctx, bad)
    with pytest.raises(_abi.KvsmcError):
        T.install(ctx, [{"dtype": "float32", "size_class": 9}])
    assert T.installed(ctx) == []


def test_autotune_small_classes(clean_tuning):
    """The autotuner times candidates on its own synthetic volumes, installs
    a table with one row per (dtype, class) asked for, and the installed
    table leaves results unchanged."""
    ctx = clean_tuning
    vols, params = _volumes(ctx)
    ref = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    table = T.autotune(ctx, dtypes=[np.float32, np.uint8], max_class=1, isovalues=2, reps=1, seed=3)
    assert [(r["dtype"], r["size_class"]) for r in table] == [
        ("float32", 0), ("float32", 1), ("uint8", 0), ("uint8", 1)]
    assert T.installed(ctx) == table
    for r in table:
        assert r["default_ms"] > 0 and 0 < r["tuned_ms"] <= r["default_ms"]
        kept = any(r[f] for f in T.FIELDS)
        assert (r["tuned_ms"] < 0.97 * r["default_ms"]) == kept or not kept
    got = extract_batch(ctx, vols, params, _abi.PATH_AUTO)
    for i in range(len(params)):
        compare(got[i], ref[i], f"tuned request {i}")
    with pytest.raises(_abi.KvsmcError):
        T.autotune(ctx, dtypes=[np.float64], max_class=0, reps=1)
    assert T.installed(ctx) == table   # a refused run keeps the table
