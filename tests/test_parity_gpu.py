"""CUDA path (libkvsmc through its C ABI) against the oracle, bit for bit.

Every case runs the whole mapper call (kvs_gb300.MarchingCubes -> C ABI ->
kernels) and the C restatement (oracle/mc_oracle.c) on the same input and
compares coords, normals, connections (bit-identical; NaN matches NaN),
colour, opacity, types, bounding box and the volume's min/max cache.
"""
import numpy as np
import pytest

from kvs_gb300 import synthetic as S
from kvs_gb300.marching_cubes import MarchingCubes, PolygonObject, StructuredVolumeObject, TransferFunction

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

MODES = [("polygon", True), ("polygon", False), ("vertex", True), ("vertex", False)]
DTYPES = [np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16, np.uint32, np.uint64,
          np.float32, np.float64]


def _volume(v, minmax=None, obj=None, grid=None, coords=None):
    vol = StructuredVolumeObject(v)
    if grid == "rectilinear":
        vol.setGridTypeToRectilinear()
        vol.setCoords(coords)
    if minmax is not None:
        vol.setMinMaxValues(*minmax)
    if obj is not None:
        vol.setMinMaxObjectCoords(*obj)
    return vol


def check(oracle_lib, ctx, v, iso, nt="polygon", dup=True, minmax=None, obj=None, grid=None, coords=None,
          tf=None):
    ntype = PolygonObject.PolygonNormal if nt == "polygon" else PolygonObject.VertexNormal
    vol = _volume(v, minmax, obj, grid, coords)
    tfunc = TransferFunction(256)
    if tf is not None:
        tfunc.setRange(*tf)
    mc = MarchingCubes(vol, iso, ntype, dup, tfunc, context=ctx)
    o = oracle_lib.marching_cubes(v, iso, nt, dup, minmax=minmax, obj_coords=obj,
                                  rect_coords=coords if grid == "rectilinear" else None,
                                  colormap=tfunc.table, tf_range=tf)
    tag = f"{v.dtype} {v.shape} iso={iso} {nt} dup={dup}"
    assert mc.isSuccess() == o["success"], tag
    assert same_bits(mc.coords(), o["coords"]), (tag, "coords", first_diff(mc.coords(), o["coords"]))
    assert same_bits(mc.normals(), o["normals"]), (tag, "normals", first_diff(mc.normals(), o["normals"]))
    assert np.array_equal(mc.connections(), o["connections"]), (tag, "connections",
                                                                first_diff(mc.connections(), o["connections"]))
    if o["coords"].size and np.isfinite(o["vol_min"]) and np.isfinite(o["vol_max"]):
        # (with a NaN value range the reference's ColorMap::at is undefined behaviour)
        assert np.array_equal(mc.colors(), o["color"]), tag
        assert np.array_equal(mc.opacities(), [255]), tag
    assert vol.hasMinMaxValues()
    assert same_bits(np.array([vol.minValue(), vol.maxValue()]), np.array([o["vol_min"], o["vol_max"]])), tag
    assert np.array_equal(mc.minObjectCoord(), o["min_obj"]) and np.array_equal(mc.maxObjectCoord(), o["max_obj"])
    assert mc.polygonType() == PolygonObject.Triangle
    return mc, o


def _field(dtype, shape, seed):
    rng = np.random.default_rng(seed)
    if np.dtype(dtype).kind == "f":
        return rng.random(shape).astype(dtype)
    info = np.iinfo(dtype)
    lo, hi = max(int(info.min), -120), min(int(info.max), 120)
    return rng.integers(lo, hi, size=shape, endpoint=True).astype(dtype)


@pytest.mark.parametrize("dtype", DTYPES, ids=[np.dtype(d).name for d in DTYPES])
@pytest.mark.parametrize("nt,dup", MODES)
def test_dtypes_and_modes(oracle_lib, kvsmc_ctx, dtype, nt, dup):
    for shape, seed in [((7, 9, 11), 1), ((13, 5, 34), 2), ((3, 40, 37), 3)]:
        v = _field(dtype, shape, seed)
        isos = [0.5, 0.3] if np.dtype(dtype).kind == "f" else [0.5, 3.0, -7.25, 10.0]
        for iso in isos:
            check(oracle_lib, kvsmc_ctx, v, iso, nt, dup)


@pytest.mark.parametrize("nt,dup", MODES[:3])
def test_smooth_fields(oracle_lib, kvsmc_ctx, nt, dup):
    b = S.to_numpy(S.gaussian_blobs((40, 48, 56), seed=5))
    check(oracle_lib, kvsmc_ctx, b, 0.5, nt, dup)
    f = S.to_numpy(S.fbm((33, 65, 70), seed=6))
    check(oracle_lib, kvsmc_ctx, f, 0.45, nt, dup)
    for dt in (np.uint8, np.uint16, np.float32):
        p = S.to_numpy(S.ellipsoid_phantom((37, 29, 45), dt, seed=7))
        lo, hi = float(p.min()), float(p.max())
        check(oracle_lib, kvsmc_ctx, p, lo + 0.37 * (hi - lo), nt, dup)


def test_config1_blobs_128(oracle_lib, kvsmc_ctx):
    """128^3 float32, 4 Gaussian blobs + noise, iso 0.5, duplication, polygon normals."""
    v = S.to_numpy(S.gaussian_blobs((128, 128, 128), seed=42))
    mc, o = check(oracle_lib, kvsmc_ctx, v, 0.5, "polygon", True)
    assert mc.coords().size // 9 > 10000


@pytest.mark.parametrize("nt,dup", MODES[:3])
def test_every_case_index(oracle_lib, kvsmc_ctx, nt, dup):
    """All 256 corner configurations, each as its own 2x2x2 volume."""
    corner_xyz = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for case in range(1, 255):
        v = np.zeros((2, 2, 2), np.float32)
        for k, (x, y, z) in enumerate(corner_xyz):
            v[z, y, x] = 1.0 if case & (1 << k) else 0.0
        check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup)
    # and one long row of cells holding every case in order
    v = np.zeros((2, 2, 257), np.float32)
    rng = np.random.default_rng(3)
    v[:] = rng.integers(0, 2, size=v.shape)
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup)


@pytest.mark.parametrize("nt,dup", MODES[:3])
def test_edge_cases(oracle_lib, kvsmc_ctx, nt, dup):
    rng = np.random.default_rng(11)
    v = rng.random((9, 10, 11)).astype(np.float32)
    # iso exactly on node values, below min, above max
    check(oracle_lib, kvsmc_ctx, v, float(v[4, 5, 6]), nt, dup)
    check(oracle_lib, kvsmc_ctx, v, -1.0, nt, dup)
    check(oracle_lib, kvsmc_ctx, v, 2.0, nt, dup)
    # isolevel that is not a float (classification in double)
    check(oracle_lib, kvsmc_ctx, v, 0.1 + 1e-12, nt, dup)
    # constant volume: Math::Equal(min, max) early exit
    check(oracle_lib, kvsmc_ctx, np.full((5, 6, 7), 3.0, np.float32), 3.0, nt, dup)
    # preset min/max narrower than the data: the clamp in interpolate_vertex
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup, minmax=(0.3, 0.7))
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup, minmax=(0.45, 0.55))
    # non-zero object coordinates: the (p + min) * scale transform
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup, obj=([1.5, -2.0, 3.25], [7.0, 9.0, 4.0]))
    # rectilinear grid (only its bounding box matters)
    coords = np.concatenate([np.linspace(0, 3, 11), np.linspace(-1, 1, 10), np.linspace(2, 5, 9)]).astype(np.float32)
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup, grid="rectilinear", coords=coords)
    # thin volumes: no cells in one axis; 2 nodes in one axis
    check(oracle_lib, kvsmc_ctx, rng.random((1, 6, 7)).astype(np.float32), 0.5, nt, dup)
    check(oracle_lib, kvsmc_ctx, rng.random((5, 1, 7)).astype(np.float32), 0.5, nt, dup)
    check(oracle_lib, kvsmc_ctx, rng.random((2, 2, 50)).astype(np.float32), 0.5, nt, dup)
    # rows whose byte length is not a multiple of 16
    check(oracle_lib, kvsmc_ctx, rng.integers(0, 255, (6, 7, 33)).astype(np.uint8), 127.5, nt, dup)
    # NaN and signed zeros in float data
    w = v.copy()
    w[2, 3, 4] = np.nan
    w[0, 0, 1] = -0.0
    check(oracle_lib, kvsmc_ctx, w, 0.5, nt, dup)
    w[0, 0, 0] = np.nan
    check(oracle_lib, kvsmc_ctx, w, 0.5, nt, dup)
    # transfer function with a preset range
    check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup, tf=(-1.0, 3.0))


def test_int_extremes(oracle_lib, kvsmc_ctx):
    """Values at the ends of the integer ranges (exact classification)."""
    rng = np.random.default_rng(5)
    for dt in (np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64):
        info = np.iinfo(dt)
        v = rng.choice(np.array([info.min, info.max, 0, 1], dtype=dt), size=(4, 5, 6))
        for iso in (0.0, 0.5, float(info.max) - 0.5, float(info.min) + 0.5, float(info.max)):
            check(oracle_lib, kvsmc_ctx, v, iso, "polygon", True)
            check(oracle_lib, kvsmc_ctx, v, iso, "polygon", False)


def test_errors_follow_the_reference(kvsmc_ctx):
    mc = MarchingCubes(context=kvsmc_ctx)
    assert mc.exec(None) is None and not mc.isSuccess()
    assert mc.exec(PolygonObject()) is None and not mc.isSuccess()
    vol = StructuredVolumeObject(np.zeros((3, 3, 3), np.float32))
    vol.setVeclen(3)
    assert mc.exec(vol) is None and not mc.isSuccess()


def test_vertex_normal_forces_shared_vertices(oracle_lib, kvsmc_ctx):
    """MarchingCubes.cpp:69-73: VertexNormal sets duplication off, and it sticks."""
    v = S.to_numpy(S.fbm((20, 21, 22), seed=8))
    mc = MarchingCubes(StructuredVolumeObject(v), 0.5, PolygonObject.VertexNormal, True, context=kvsmc_ctx)
    assert mc.connections().size > 0
    mc.setNormalType(PolygonObject.PolygonNormal)
    mc.exec(StructuredVolumeObject(v))
    o = oracle_lib.marching_cubes(v, 0.5, "polygon", False)
    assert o["connections"].size > 0
    assert np.array_equal(mc.connections(), o["connections"])


@pytest.mark.parametrize("width", [4097, 4098, 4500])
def test_widths_at_and_past_the_streaming_limit(oracle_lib, kvsmc_ctx, width):
    """Rows of up to 4097 nodes take the streaming kernels, wider ones the
    gather kernels: the same bits either way, all three modes."""
    v = S.to_numpy(S.fbm((4, 5, width), seed=width))
    for nt, dup in MODES[:3]:
        check(oracle_lib, kvsmc_ctx, v, 0.5, nt, dup)
