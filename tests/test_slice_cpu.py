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
