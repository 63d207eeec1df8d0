"""The binary STL restatement (oracle/export.py) against files written by the
reference PolygonExporter<kvs::Stl> + Stl::write_binary (tests/golden/stl.npz),
byte for byte, and the format's invariants."""
import json
import os

import numpy as np
import pytest

from oracle import export as E
from oracle import ref

from .helpers import GOLDEN_DIR


def stl_fixtures():
    man = json.load(open(os.path.join(GOLDEN_DIR, "stl.json")))
    arr = np.load(os.path.join(GOLDEN_DIR, "stl.npz"))
    return man, arr


def test_restatement_matches_reference_files():
    man, arr = stl_fixtures()
    assert len(man) >= 8
    for e in man:
        k = e["case"]
        got = E.stl_binary(arr[f"{k}__coords"], arr[f"{k}__normals"], arr[f"{k}__connections"], e["normal_type_out"])
        want = arr[f"{k}__stl"].tobytes()
        assert got == want, k
        assert len(want) == 84 + 50 * e["ntriangles"], k
        assert want[:16] == b"Generated by KVS" and want[16:80] == bytes(64), k


def test_record_layout():
    coords = np.arange(18, dtype=np.float32)
    normals = np.array([1, 2, 3, -1, -2, -3], np.float32)
    b = E.stl_binary(coords, normals, np.zeros(0, np.uint32), E.POLYGON_NORMAL)
    assert np.frombuffer(b[80:84], "<u4")[0] == 2
    r = np.frombuffer(b[84:], E.RECORD)
    assert np.array_equal(r["n"][1], [-1, -2, -3]) and np.array_equal(r["c"][1], np.arange(9, 18))
    assert np.all(r["attr"] == 0)


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_fixtures_are_current():
    man, arr = stl_fixtures()
    for e in man:
        k = e["case"]
        b = ref.marching_cubes_stl(arr[f"{k}__input"], e["isolevel"], e["normal_type"], e["duplication"])
        assert b == arr[f"{k}__stl"].tobytes(), k
