"""Binary PLY export: the restatement (oracle/export.py ply_binary) against
files written by the reference PolygonExporter<kvs::Ply> + Ply::write
(tests/golden/ply.npz), byte for byte; the library's header writer against
those files; the mirror's mode choice and refusals (no GPU needed)."""
import ctypes
import json
import os

import numpy as np
import pytest

from kvs_gb300.export import PolygonExporterPly, ply_modes
from kvs_gb300.marching_cubes import PolygonObject
from oracle import export as E

from .helpers import GOLDEN_DIR


def ply_fixtures():
    return json.load(open(os.path.join(GOLDEN_DIR, "ply.json"))), np.load(os.path.join(GOLDEN_DIR, "ply.npz"))


def polygon_of(arr, e):
    p = PolygonObject()
    k = e["case"]
    p._coords = arr[f"{k}__coords"]
    p._colors = arr[f"{k}__colors"]
    p._normals = arr[f"{k}__normals"]
    p._polygon_type = PolygonObject.Triangle
    p._color_type = PolygonObject.VertexColor if e["color_type"] == "vertex" else PolygonObject.PolygonColor
    p._normal_type = PolygonObject.VertexNormal if e["normal_type"] == "vertex" else PolygonObject.PolygonNormal
    return p


def test_restatement_matches_reference_files():
    man, arr = ply_fixtures()
    assert len(man) >= 6
    for e in man:
        k = e["case"]
        b = E.ply_binary(arr[f"{k}__coords"], arr[f"{k}__colors"], arr[f"{k}__normals"], e["color_type"],
                         e["normal_type"])
        assert b == arr[f"{k}__file"].tobytes(), k


def test_modes():
    man, arr = ply_fixtures()
    want = {"mc_dup": (1, 1), "slice": (2, 1), "vertex_normals": (2, 2), "bare": (0, 0),
            "one_colour_no_normals": (1, 0), "empty": (0, 0)}
    for e in man:
        assert ply_modes(polygon_of(arr, e)) == want[e["case"]], e["case"]


def test_refusals(capsys):
    p = PolygonObject()
    p._coords = np.zeros(9, np.float32)
    p._connections = np.array([0, 1, 2], np.uint32)
    p._polygon_type = PolygonObject.Triangle
    with pytest.raises(ValueError):
        ply_modes(p)
    p._connections = np.zeros(0, np.uint32)
    p._colors = np.zeros(9, np.uint8)
    p._color_type = PolygonObject.PolygonColor
    with pytest.raises(ValueError):
        ply_modes(p)
    ex = PolygonExporterPly(p)
    assert ex.isSuccess()
    assert not ex.write("/nonexistent/x.ply")          # ASCII (the reference default) is not provided
    assert "ASCII PLY" in capsys.readouterr().err
    assert PolygonExporterPly().exec(None) is None


def test_library_header_matches_reference_files():
    """kvsmc_ply_header and kvsmc_ply_record_bytes (host code in libkvsmc.so,
    no GPU needed) give the reference file's header bytes and its size."""
    from kvs_gb300 import _abi
    lib = _abi.load()
    man, arr = ply_fixtures()
    for e in man:
        k = e["case"]
        f = arr[f"{k}__file"].tobytes()
        nv = arr[f"{k}__coords"].size // 3
        cmode, nmode = ply_modes(polygon_of(arr, e))
        need = lib.kvsmc_ply_header(nv, cmode, nmode, None, 0)
        assert need > 0, k
        buf = ctypes.create_string_buffer(need + 1)
        assert lib.kvsmc_ply_header(nv, cmode, nmode, buf, need + 1) == need, k
        head = buf.raw[:need]
        assert f[:need] == head and head.endswith(b"end_header\n"), k
        assert len(f) == need + nv * lib.kvsmc_ply_record_bytes(cmode, nmode), k
    small = ctypes.create_string_buffer(b"x" * 8)
    assert lib.kvsmc_ply_header(3, 1, 1, small, 8) > 8
    assert small.raw == b"x" * 8 + b"\0"                 # too small a buffer is left untouched
