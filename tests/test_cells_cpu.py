"""Unstructured marching mappers on the CPU: the numpy restatement
(oracle/cells.py) against the fixtures made from the reference
MarchingTetrahedra / Hexahedra / Pyramid / Prism (tests/golden/cells.npz),
bit for bit; the fixtures against the reference where it is built; the
pyramid's ambiguous cases are covered; and the mirror's host-side checks."""
import json
import os

import numpy as np
import pytest

from kvs_gb300 import marching_cells as mcells
from oracle import cells as ocells
from oracle import ref

from . import cell_meshes as cm
from .helpers import GOLDEN_DIR, first_diff, same_bits


def cells_fixtures():
    return json.load(open(os.path.join(GOLDEN_DIR, "cells.json"))), np.load(os.path.join(GOLDEN_DIR, "cells.npz"))


def case_inputs(arr, e):
    c = e["case"]
    return arr[f"{c}__values"], arr[f"{c}__coords"], arr[f"{c}__connections"]


def extracts(e):
    """Whether the reference extracts triangles for this run (not without
    duplicated vertices, which VertexNormal forces)."""
    return e["duplication"] and e["normal_type"] == "polygon"


def test_fixture_shapes():
    man, arr = cells_fixtures()
    assert len(man) >= 100
    for ct in range(4):
        assert sum(1 for e in man if e["cell_type"] == ct and e["ntriangles"] > 0) >= 15
    for e in man:
        k, n = e["key"], e["ntriangles"]
        assert arr[f"{k}__coords"].size == 9 * n and arr[f"{k}__normals"].size == 3 * n, k
        assert arr[f"{k}__connections"].size == 0, k
        assert arr[f"{k}__colors"].size == (3 if n else 0), k
        assert not e["success"], k            # the mappers never set success
        if not extracts(e):
            assert n == 0, k


def test_oracle_matches_reference_fixtures():
    man, arr = cells_fixtures()
    for e in man:
        k = e["key"]
        v, xyz, conn = case_inputs(arr, e)
        o = ocells.marching_cells(e["cell_type"], v, xyz, conn, e["iso"], e["minmax"])
        want = arr[f"{k}__vol_minmax"]
        if e["minmax"] is None:
            assert same_bits(np.array([o["vmin"], o["vmax"]]), want), (k, o["vmin"], o["vmax"], want)
        if not extracts(e):
            continue
        for f in ("coords", "normals"):
            assert same_bits(o[f], arr[f"{k}__{f}"]), (k, f, first_diff(o[f], arr[f"{k}__{f}"]))


def test_oracle_bounding_box_matches_reference():
    man, arr = cells_fixtures()
    for e in man:
        v, xyz, conn = case_inputs(arr, e)
        lo, hi = ocells.min_max_coords(xyz, conn)
        assert np.array_equal(lo, np.float32(e["min_obj"])) and np.array_equal(hi, np.float32(e["max_obj"])), e["key"]


def test_mirror_bounding_box_matches_reference():
    man, arr = cells_fixtures()
    for e in man[::5]:
        v, xyz, conn = case_inputs(arr, e)
        vol = mcells.UnstructuredVolumeObject(mcells.MAPPERS_BY_ABI[e["cell_type"]].CELL, v.size, conn.shape[0],
                                              1, xyz, conn, v)
        vol.updateMinMaxCoords()
        assert np.array_equal(vol.minObjectCoord(), np.float32(e["min_obj"])), e["key"]
        assert np.array_equal(vol.maxExternalCoord(), np.float32(e["max_ext"])), e["key"]


def test_pyramid_ambiguous_cases_covered():
    """Cases 10, 11, 20, 21 go both ways (and E == 0 occurs) in the fixtures."""
    man, arr = cells_fixtures()
    seen, zero = set(), 0
    for e in man:
        if e["cell_type"] != 2 or e["minmax"] is not None:
            continue
        v, xyz, conn = case_inputs(arr, e)
        if conn.size == 0:
            continue
        vals = v[conn.astype(np.int64)].astype(np.float64)
        case = sum(((vals[:, k] > e["iso"]).astype(np.int64) << k) for k in range(5))
        v1, v2, v3, v4 = vals[:, 1], vals[:, 2], vals[:, 3], vals[:, 4]
        with np.errstate(all="ignore"):
            E = (e["iso"] - (v1 + v2 + v3 + v4) / 4) * ((v1 - v2 + v3 - v4) / 4) + \
                ((-v1 + v2 + v3 - v4) / 4) * ((-v1 - v2 + v3 + v4) / 4)
        for c in (10, 11, 20, 21):
            m = case == c
            if np.any(m & (E < 0)):
                seen.add((c, "-"))
            if np.any(m & (E >= 0)):
                seen.add((c, "+"))
            zero += int(np.sum(m & (E == 0)))
    assert seen == {(c, s) for c in (10, 11, 20, 21) for s in "+-"}, seen
    assert zero > 0


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_fixtures_are_current():
    man, arr = cells_fixtures()
    for e in man[::3]:
        v, xyz, conn = case_inputs(arr, e)
        r = ref.marching_cells(e["cell_type"], v, xyz, conn, e["iso"], form=e["form"], normal_type=e["normal_type"],
                               duplication=e["duplication"], minmax=e["minmax"], tf_range=e["tf_range"])
        for f in ("coords", "normals", "colors", "opacities"):
            assert same_bits(r[f], arr[f"{e['key']}__{f}"]), (e["key"], f)


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_oracle_matches_reference_on_grids():
    """Larger jittered grids of each cell type, several isolevels."""
    for ct in range(4):
        xyz, conn = cm.grid(ct, 14, 12, 10, seed=7 + ct)
        v = cm.sphere_values(xyz, (6.1, 5.3, 4.7))
        for iso in (2.5, 4.0):
            r = ref.marching_cells(ct, v, xyz, conn, iso)
            o = ocells.marching_cells(ct, v, xyz, conn, iso)
            assert r["coords"].size > 0
            assert same_bits(o["coords"], r["coords"]) and same_bits(o["normals"], r["normals"]), (ct, iso)


def test_mirror_checks_without_gpu(capsys):
    """exec's checks and messages run before any GPU call."""
    assert mcells.MarchingTetrahedra().exec(None) is None
    assert "Input object is NULL." in capsys.readouterr().err
    assert mcells.MarchingPrism().exec(object()) is None
    assert "Input object is not unstructured volume object." in capsys.readouterr().err
    vol = mcells.UnstructuredVolumeObject(mcells.UnstructuredVolumeObject.Hexahedra, 8, 1, 3)
    assert mcells.MarchingHexahedra().exec(vol) is None
    assert "Input volume is not sclar field data." in capsys.readouterr().err
    vol.setVeclen(1)
    for m, msg in ((mcells.MarchingTetrahedra, "tetrahedra"), (mcells.MarchingPyramid, "pyramid"),
                   (mcells.MarchingPrism, "prism")):
        mapper = m()
        assert mapper.exec(vol) is None and mapper.isFailure()
        assert f"Input volume is not {msg}-cell data." in capsys.readouterr().err
    assert mcells.UnstructuredVolumeObject(mcells.UnstructuredVolumeObject.Pyramid).numberOfCellNodes() == 5


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_oracle_matches_reference_on_random_meshes_with_ties():
    """Random connectivity (repeated and degenerate nodes, cells in any
    orientation) with node values on a coarse lattice so that many equal the
    isolevel exactly; each cell type, value type and isolevel."""
    for ct in range(4):
        xyz, conn = cm.random_mesh(ct, 300, 900, seed=31 + ct)
        rng = np.random.default_rng(5 + ct)
        lattice = rng.integers(0, 9, 300)
        for dt in (np.float32, np.int16, np.uint8):
            v = lattice.astype(dt)
            for iso in (3.0, 4.0, 4.5):
                r = ref.marching_cells(ct, v, xyz, conn, iso)
                o = ocells.marching_cells(ct, v, xyz, conn, iso)
                assert r["coords"].size > 0, (ct, dt, iso)
                assert same_bits(o["coords"], r["coords"]), (ct, dt, iso, first_diff(o["coords"], r["coords"]))
                assert same_bits(o["normals"], r["normals"]), (ct, dt, iso)


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_oracle_matches_reference_on_full_range_values():
    """All ten value types with values across the type's whole range (64-bit
    integers that doubles round, the volume's min/max clamp at the extremes),
    isolevels inside the range."""
    rng = np.random.default_rng(29)
    for ct in range(4):
        xyz, conn = cm.grid(ct, 9, 8, 7, seed=13 + ct)
        for dt in (np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64,
                   np.float32, np.float64):
            if np.issubdtype(dt, np.integer):
                info = np.iinfo(dt)
                v = rng.integers(info.min, info.max, xyz.shape[0], dtype=dt, endpoint=True)
            else:
                v = (rng.standard_normal(xyz.shape[0]) * 1e30).astype(dt)
            iso = float(v.min()) * 0.25 + float(v.max()) * 0.75
            r = ref.marching_cells(ct, v, xyz, conn, iso)
            o = ocells.marching_cells(ct, v, xyz, conn, iso)
            assert r["coords"].size > 0, (ct, dt)
            assert same_bits(o["coords"], r["coords"]), (ct, dt, first_diff(o["coords"], r["coords"]))
            assert same_bits(o["normals"], r["normals"]), (ct, dt)
