"""kvs::Isosurface's structured branch (Isosurface.cpp): the fixtures made from
the reference build (tests/golden/isosurface.npz) against the oracle's
restatement of the rules the wrapper adds over MarchingCubes (default
isolevel (max + min) * 0.5 from the volume's min/max cache, VertexNormal
forcing shared vertices, the transfer function of each constructor form),
and, where the reference build exists, the reference Isosurface against the
reference MarchingCubes and against the fixtures."""
import json
import os

import numpy as np
import pytest

from oracle import ref

from .helpers import GOLDEN_DIR, first_diff, same_bits


def fixtures():
    man = json.load(open(os.path.join(GOLDEN_DIR, "isosurface.json")))
    arr = np.load(os.path.join(GOLDEN_DIR, "isosurface.npz"))
    return man, arr


def effective(e, v, minmax_fn):
    """(isolevel, duplication) the reference Isosurface hands to MarchingCubes."""
    if e["form"] == 0:
        mn, mx = e["minmax"] if e["minmax"] else minmax_fn(v)
        iso = (mx + mn) * 0.5
    else:
        iso = e["isolevel"]
    dup = e["duplication"] and e["normal_type"] != "vertex"
    return iso, dup


def test_oracle_restates_isosurface(oracle_lib):
    man, arr = fixtures()
    cmap = np.load(os.path.join(GOLDEN_DIR, "golden.npz"))["colormap256"]
    assert len(man) >= 15
    for e in man:
        v = arr[f"{e['case']}__input"]
        iso, dup = effective(e, v, oracle_lib.minmax)
        o = oracle_lib.marching_cubes(v, iso, e["normal_type"], dup, minmax=e["minmax"], colormap=cmap,
                                      tf_range=e["tf_range"] if e["form"] == 2 else None)
        k = e["key"]
        assert same_bits(o["coords"], arr[f"{k}__coords"]), (k, first_diff(o["coords"], arr[f"{k}__coords"]))
        assert same_bits(o["normals"], arr[f"{k}__normals"]), k
        assert np.array_equal(o["connections"], arr[f"{k}__connections"]), k
        if arr[f"{k}__coords"].size:
            assert np.array_equal(o["color"], arr[f"{k}__colors"]), k
        assert o["vol_min"] == e["vol_min"] or (np.isnan(o["vol_min"]) and np.isnan(e["vol_min"])), k


@pytest.mark.skipif(not ref.available(), reason="needs the reference build (oracle/_ref)")
def test_reference_isosurface_is_marching_cubes_and_fixtures_are_current():
    man, arr = fixtures()
    for e in man:
        v = arr[f"{e['case']}__input"]
        r = ref.isosurface(v, e["form"], e["isolevel"], e["normal_type"], e["duplication"], minmax=e["minmax"],
                           tf_range=e["tf_range"])
        k = e["key"]
        for f in ("coords", "normals", "connections", "colors", "opacities"):
            assert same_bits(r[f], arr[f"{k}__{f}"]), (k, f)
        assert not r["success"]   # the reference never sets Isosurface's success flag (MapperBase.cpp:23)
        iso, dup = effective(e, v, lambda x: (r["vol_min"], r["vol_max"]))
        m = ref.marching_cubes(v, iso, e["normal_type"], dup, minmax=e["minmax"],
                               tf_range=e["tf_range"] if e["form"] == 2 else None)
        assert m["success"]
        for f in ("coords", "normals", "connections", "colors", "opacities"):
            assert same_bits(r[f], m[f]), (k, f)
        assert (r["polygon_type"], r["normal_type"], r["color_type"]) == (
            m["polygon_type"], m["normal_type"], m["color_type"]), k
        assert np.array_equal(r["min_obj"], m["min_obj"]) and np.array_equal(r["max_ext"], m["max_ext"]), k
