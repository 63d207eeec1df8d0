"""The ASCII STL and KVSML polygon restatements (oracle/export.py) against the
files the reference's own writers made (tests/golden/exports.npz, written by
PolygonExporter<kvs::Stl> with the Ascii file type and by
PolygonExporter<kvs::KVSMLPolygonObject> with each writing data type), on the
oracle's MarchingCubes results of the same inputs."""
import json
import os

import numpy as np
import pytest

from oracle import export as oexp

HERE = os.path.dirname(os.path.abspath(__file__))
MAN = json.load(open(os.path.join(HERE, "golden", "exports.json")))
ARR = np.load(os.path.join(HERE, "golden", "exports.npz"))
TYPES = {"kvsml_ascii": 0, "kvsml_external_ascii": 1, "kvsml_external_binary": 2}


def _mesh(oracle_lib, e):
    v = ARR[f"{e['case']}__input"]
    return oracle_lib.marching_cubes(v, e["isolevel"], e["normal_type"], e["duplication"],
                                     colormap=None)


@pytest.mark.parametrize("e", MAN, ids=[e["case"] for e in MAN])
def test_stl_ascii_restatement(oracle_lib, e):
    o = _mesh(oracle_lib, e)
    nt = oexp.VERTEX_NORMAL if e["normal_type"] == "vertex" else oexp.POLYGON_NORMAL
    got = oexp.stl_ascii(o["coords"], o["normals"], o["connections"], nt)
    (fn,) = e["files"]["stl_ascii"]
    assert got == ARR[f"{e['case']}__stl_ascii__{fn}"].tobytes()


@pytest.mark.parametrize("e", MAN, ids=[e["case"] for e in MAN])
def test_kvsml_restatement(oracle_lib, e):
    from kvs_gb300.marching_cubes import TransferFunction
    v = ARR[f"{e['case']}__input"]
    o = oracle_lib.marching_cubes(v, e["isolevel"], e["normal_type"], e["duplication"],
                                  colormap=TransferFunction(256).table)
    normal_type = "vertex" if e["normal_type"] == "vertex" else "polygon"
    color = o["color"] if o["coords"].size else None
    for fmt, wt in TYPES.items():
        files = oexp.kvsml_polygon(e["case"], wt, o["coords"], o["normals"], o["connections"], normal_type,
                                   color, np.array([255], np.uint8))
        assert sorted(files) == e["files"][fmt], (fmt, sorted(files))
        for fn, data in files.items():
            assert data == ARR[f"{e['case']}__{fmt}__{fn}"].tobytes(), (fmt, fn)
