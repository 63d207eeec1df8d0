"""kvs::SlicePlane fixtures (tests/golden/slice.npz, made from the reference
build): current against the reference where it is built, and the format's
invariants (9 floats and 9 colour bytes per triangle, one normal each)."""
import json
import os

import numpy as np
import pytest

from oracle import ref

from .helpers import GOLDEN_DIR, same_bits


def slice_fixtures():
    return json.load(open(os.path.join(GOLDEN_DIR, "slice.json"))), np.load(os.path.join(GOLDEN_DIR, "slice.npz"))


def test_fixture_shapes():
    man, arr = slice_fixtures()
    assert len(man) >= 15 and any(e["ntriangles"] == 0 for e in man)
    for e in man:
        k, n = e["key"], e["ntriangles"]
        assert arr[f"{k}__coords"].size == 9 * n and arr[f"{k}__colors"].size == 9 * n, k
        assert arr[f"{k}__normals"].size == 3 * n, k
        assert list(arr[f"{k}__opacities"]) == [255], k
        assert not e["success"]   # the reference never sets SlicePlane's success flag


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_fixtures_are_current():
    man, arr = slice_fixtures()
    for e in man:
        v = arr[f"{e['case']}__input"]
        r = ref.slice_plane(v, coefficients=e["coefficients"], point=e["point"], normal=e["normal"],
                            tf_range=e["tf_range"])
        for f in ("coords", "normals", "colors", "opacities"):
            assert same_bits(r[f], arr[f"{e['key']}__{f}"]), (e["key"], f)


def _minmax(v):
    return float(v.min()), float(v.max())


def test_restatement_matches_reference_fixtures():
    """oracle/slice.py against the reference's files, bit for bit: all ten
    value types, both plane forms, planes through nodes, an empty slice."""
    from oracle import slice as OS
    from .test_slice_cells_cpu import plane_of, tf_range_of
    from .helpers import first_diff, golden
    table = golden()[1]["colormap256"]
    man, arr = slice_fixtures()
    for e in man:
        k = e["key"]
        v = arr[f"{e['case']}__input"]
        lo, hi = tf_range_of(e, v, _minmax(v))
        c, rgb, n = OS.slice_plane(v, plane_of(e), table, lo, hi)
        assert same_bits(c, arr[f"{k}__coords"]), (k, first_diff(c, arr[f"{k}__coords"]))
        assert np.array_equal(rgb, arr[f"{k}__colors"]), k
        assert same_bits(n, arr[f"{k}__normals"]), k


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_restatement_matches_reference_on_larger_volumes():
    """Rows longer than a warp, several value types, axis planes through node
    layers and oblique planes; the reference run live on the same inputs."""
    from oracle import slice as OS
    from .helpers import first_diff, golden
    table = golden()[1]["colormap256"]
    rng = np.random.default_rng(11)
    base = rng.random((23, 31, 70))
    for dt in (np.float32, np.uint16, np.int32, np.float64):
        v = (base * 1000 - (500 if np.issubdtype(dt, np.signedinteger) else 0)).astype(dt)
        lo, hi = np.float32(v.min()), np.float32(v.max())
        for coef in ((1, 0, 0, -33), (0, 0, 1, -11.5), (0.3, -0.55, 0.78, -4.2), (0.05, 0.02, -1, 7)):
            r = ref.slice_plane(v, coefficients=list(coef), point=None, normal=None, tf_range=(float(lo), float(hi)))
            c, rgb, n = OS.slice_plane(v, coef, table, lo, hi)
            assert r["coords"].size > 0, (dt, coef)
            assert same_bits(c, r["coords"]), (dt, coef, first_diff(c, r["coords"]))
            assert np.array_equal(rgb, r["colors"]), (dt, coef)
            assert same_bits(n, r["normals"]), (dt, coef)


def large_slice_cases():
    """Seeded volumes for the GPU parity test (and their CPU pin): rows of
    4500 nodes (past a warp's and a block's width), a plane through a whole
    cell layer (every cell of the layer cut), a plane nearly parallel to the
    rows, a plane through node diagonals of a uint8 volume, an int16 volume."""
    rng = np.random.default_rng(3)
    v = rng.random((30, 41, 4500)).astype(np.float32)
    yield "f32_layer", v, (0, 0, 1, -11.5)
    yield "f32_shallow", v, (0.01, 0.3, -1, 9.2)
    yield "u8_diagonal", rng.integers(0, 256, (97, 130, 200)).astype(np.uint8), (1, 1, -1, -50)
    yield "i16_tilted", rng.integers(-3000, 3000, (64, 64, 64)).astype(np.int16), (0.002, -1, 0.001, 31.7)


def default_tf_range(v):
    """MapperBase::setRange with a default transfer function (no NaN values):
    the volume's min/max as doubles, then the float range."""
    if v.dtype == np.int8:
        return np.float32(-128), np.float32(127)
    if v.dtype == np.uint8:
        return np.float32(0), np.float32(255)
    return np.float32(float(v.min())), np.float32(float(v.max()))


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_restatement_matches_reference_on_gpu_test_cases():
    from oracle import slice as OS
    from .helpers import first_diff, golden
    table = golden()[1]["colormap256"]
    for name, v, coef in large_slice_cases():
        lo, hi = default_tf_range(v)
        r = ref.slice_plane(v, coefficients=list(coef), point=None, normal=None, tf_range=(float(lo), float(hi)))
        c, rgb, n = OS.slice_plane(v, coef, table, lo, hi)
        assert r["coords"].size > 0, name
        assert same_bits(c, r["coords"]), (name, first_diff(c, r["coords"]))
        assert np.array_equal(rgb, r["colors"]), name
        assert same_bits(n, r["normals"]), name


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_restatement_matches_reference_with_object_coords():
    """A volume whose object coordinates are preset (scale_coord with a
    non-zero origin and non-unit cell sizes)."""
    from oracle import slice as OS
    from .helpers import first_diff, golden
    table = golden()[1]["colormap256"]
    v = np.random.default_rng(19).random((13, 17, 40)).astype(np.float32)
    lo, hi = default_tf_range(v)
    for obj in (([1.5, -2.0, 0.25], [9.0, 3.3, 7.0]), ([-10, -10, -10], [10, 10, 10])):
        for coef in ((0, 0, 1, -6.5), (0.4, -0.2, 0.6, -5.1)):
            r = ref.slice_plane(v, coefficients=list(coef), point=None, normal=None,
                                tf_range=(float(lo), float(hi)), obj_coords=obj)
            c, rgb, n = OS.slice_plane(v, coef, table, lo, hi, min_coord=obj[0], max_coord=obj[1])
            assert r["coords"].size > 0 and np.array_equal(r["min_obj"], np.float32(obj[0])), (obj, coef)
            assert same_bits(c, r["coords"]), (obj, coef, first_diff(c, r["coords"]))
            assert np.array_equal(rgb, r["colors"]), (obj, coef)
            assert same_bits(n, r["normals"]), (obj, coef)


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_restatement_matches_reference_on_full_range_values():
    """All ten value types with values across the type's whole range, so that
    the difference values[i1] - values[i0] wraps in the narrow and 64-bit
    integer types as it does in C++ (colour from the wrapped difference)."""
    from oracle import slice as OS
    from .helpers import first_diff, golden
    table = golden()[1]["colormap256"]
    rng = np.random.default_rng(23)
    shape = (11, 14, 37)
    for dt in (np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64,
               np.float32, np.float64):
        if np.issubdtype(dt, np.integer):
            info = np.iinfo(dt)
            v = rng.integers(info.min, info.max, shape, dtype=dt, endpoint=True)
        else:
            v = (rng.standard_normal(shape) * 1e6).astype(dt)
        lo, hi = default_tf_range(v)
        for coef in ((0.3, -0.55, 0.78, -4.2), (0, 1, 0, -6)):
            r = ref.slice_plane(v, coefficients=list(coef), point=None, normal=None, tf_range=(float(lo), float(hi)))
            c, rgb, n = OS.slice_plane(v, coef, table, lo, hi)
            assert r["coords"].size > 0, (dt, coef)
            assert same_bits(c, r["coords"]), (dt, coef, first_diff(c, r["coords"]))
            assert np.array_equal(rgb, r["colors"]), (dt, coef, np.flatnonzero(rgb != r["colors"])[:5])
            assert same_bits(n, r["normals"]), (dt, coef)
