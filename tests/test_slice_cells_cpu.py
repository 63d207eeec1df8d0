"""kvs::SlicePlane on unstructured volumes, on the CPU: the numpy restatement
(oracle/cells.py slice_cells) against the fixtures made from the reference
SlicePlane (tests/golden/slice_cells.npz), bit for bit, including nodes that
lie exactly on the plane, all ten value types and both plane forms."""
import json
import os

import numpy as np
import pytest

from oracle import cells as ocells
from oracle import ref

from .helpers import GOLDEN_DIR, first_diff, golden, same_bits


def slice_cells_fixtures():
    return (json.load(open(os.path.join(GOLDEN_DIR, "slice_cells.json"))),
            np.load(os.path.join(GOLDEN_DIR, "slice_cells.npz")))


def case_inputs(arr, e):
    c = e["case"]
    return arr[f"{c}__values"], arr[f"{c}__coords"], arr[f"{c}__connections"]


def plane_of(e):
    """SlicePlane::setPlane: coefficients, or (normal, -point.dot(normal)) in float."""
    f32 = np.float32
    if e["coefficients"] is not None:
        return np.asarray(e["coefficients"], f32)
    p, n = np.asarray(e["point"], f32), np.asarray(e["normal"], f32)
    dot = f32(f32(f32(p[0] * n[0]) + f32(p[1] * n[1])) + f32(p[2] * n[2]))
    return np.array([n[0], n[1], n[2], -dot], f32)


def tf_range_of(e, v, vol_minmax):
    """MapperBase::setRange for the fixtures' default transfer function."""
    f32 = np.float32
    if e["tf_range"] is not None:
        return f32(e["tf_range"][0]), f32(e["tf_range"][1])
    if v.dtype == np.int8:
        return f32(-128), f32(127)
    if v.dtype == np.uint8:
        return f32(0), f32(255)
    lo, hi = f32(vol_minmax[0]), f32(vol_minmax[1])
    return (lo, hi + f32(1)) if abs(float(lo) - float(hi)) < 1e-6 else (lo, hi)


def test_fixture_shapes():
    man, arr = slice_cells_fixtures()
    assert len(man) >= 60
    for e in man:
        k, n = e["key"], e["ntriangles"]
        assert arr[f"{k}__coords"].size == 9 * n and arr[f"{k}__colors"].size == 9 * n, k
        assert arr[f"{k}__normals"].size == 3 * n, k
        assert list(arr[f"{k}__opacities"]) == [255], k
        assert not e["success"], k
        assert (e["polygon_type"], e["color_type"], e["normal_type"]) == (3, 0, 1), k


def test_oracle_matches_reference_fixtures():
    man, arr = slice_cells_fixtures()
    table = golden()[1]["colormap256"]
    for e in man:
        k = e["key"]
        v, xyz, conn = case_inputs(arr, e)
        lo, hi = tf_range_of(e, v, arr[f"{k}__vol_minmax"])
        c, rgb, n = ocells.slice_cells(e["cell_type"], v, xyz, conn, plane_of(e), table, lo, hi)
        assert same_bits(c, arr[f"{k}__coords"]), (k, first_diff(c, arr[f"{k}__coords"]))
        assert np.array_equal(rgb, arr[f"{k}__colors"]), k
        assert same_bits(n, arr[f"{k}__normals"]), k
        if conn.size:
            lo_v, hi_v = ocells.minmax(v, conn, e["cell_type"])
            assert same_bits(np.array([lo_v, hi_v]), arr[f"{k}__vol_minmax"]), k


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_fixtures_are_current():
    man, arr = slice_cells_fixtures()
    for e in man[::4]:
        v, xyz, conn = case_inputs(arr, e)
        r = ref.slice_cells(e["cell_type"], v, xyz, conn, coefficients=e["coefficients"], point=e["point"],
                            normal=e["normal"], tf_range=e["tf_range"])
        for f in ("coords", "normals", "colors"):
            assert same_bits(r[f], arr[f"{e['key']}__{f}"]), (e["key"], f)


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_oracle_matches_reference_on_random_meshes():
    """Random connectivity (repeated nodes, any orientation) with node
    coordinates on a half-unit lattice, cut by axis planes through lattice
    values (many nodes exactly on the plane) and by an oblique plane."""
    from . import cell_meshes as cm
    table = golden()[1]["colormap256"]
    for ct in range(4):
        xyz, conn = cm.random_mesh(ct, 300, 900, seed=41 + ct)
        xyz = (np.round(xyz * 2) / 2).astype(np.float32)
        v = np.random.default_rng(ct).uniform(-1, 1, 300).astype(np.float32)
        lo, hi = np.float32(-1.5), np.float32(2.0)
        for coef in ((1, 0, 0, -0.5), (0, 1, 0, 1.0), (0, 0, -1, 0), (0.3, -0.7, 0.2, 0.1)):
            r = ref.slice_cells(ct, v, xyz, conn, coefficients=coef, point=None, normal=None,
                                tf_range=(float(lo), float(hi)))
            c, rgb, n = ocells.slice_cells(ct, v, xyz, conn, np.asarray(coef, np.float32), table, lo, hi)
            assert r["coords"].size > 0, (ct, coef)
            assert same_bits(c, r["coords"]), (ct, coef, first_diff(c, r["coords"]))
            assert np.array_equal(rgb, r["colors"]), (ct, coef)
            assert same_bits(n, r["normals"]), (ct, coef)
