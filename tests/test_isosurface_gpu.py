"""kvs_gb300.isosurface.Isosurface (kvs::Isosurface with its structured branch
on the GPU) against the fixtures made from the reference kvs::Isosurface,
bit for bit: every constructor form, VertexNormal, preset and device-scanned
min/max, NaN values, a constant volume."""
import numpy as np
import pytest

from kvs_gb300.isosurface import Isosurface
from kvs_gb300.marching_cubes import PolygonObject, StructuredVolumeObject, TransferFunction

from .helpers import first_diff, same_bits
from .test_isosurface_cpu import fixtures

pytestmark = pytest.mark.gpu


def _run(e, v, ctx):
    vol = StructuredVolumeObject(v)
    if e["minmax"]:
        vol.setMinMaxValues(*e["minmax"])
    nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
    if e["form"] == 0:
        return Isosurface(vol, normal_type=nt, context=ctx), vol
    if e["form"] == 1:
        return Isosurface(vol, e["isolevel"], nt, context=ctx), vol
    tf = TransferFunction(256)
    if e["tf_range"]:
        tf.setRange(*e["tf_range"])
    return Isosurface(vol, e["isolevel"], nt, e["duplication"], tf, context=ctx), vol


def test_isosurface_matches_reference_fixtures(kvsmc_ctx):
    man, arr = fixtures()
    for e in man:
        v = arr[f"{e['case']}__input"]
        iso, vol = _run(e, v, kvsmc_ctx)
        k = e["key"]
        assert iso.isSuccess() == e["success"], k        # never set true, as in the reference
        assert same_bits(iso.coords(), arr[f"{k}__coords"]), (k, first_diff(iso.coords(), arr[f"{k}__coords"]))
        assert same_bits(iso.normals(), arr[f"{k}__normals"]), (k, first_diff(iso.normals(), arr[f"{k}__normals"]))
        assert np.array_equal(iso.connections(), arr[f"{k}__connections"]), k
        assert np.array_equal(iso.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(iso.opacities(), arr[f"{k}__opacities"]), k
        assert (iso.polygonType(), iso.normalType(), iso.colorType()) == (
            e["polygon_type"], e["normal_type_out"], e["color_type"]), k
        assert np.array_equal(iso.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(iso.maxExternalCoord(), np.float32(e["max_ext"])), k
        # the volume's min/max cache, filled by the device scan where not preset
        assert same_bits(np.float64([vol.minValue(), vol.maxValue()]), np.float64([e["vol_min"], e["vol_max"]])), k


def test_isosurface_rejects_like_the_reference(kvsmc_ctx, capsys):
    iso = Isosurface(context=kvsmc_ctx)
    assert iso.exec(None) is None and iso.isFailure()
    assert iso.exec(np.zeros((3, 3, 3))) is None
    vec = StructuredVolumeObject(np.zeros((4, 4, 4, 3), np.float32).reshape(-1), resolution=(4, 4, 4), veclen=3)
    assert iso.exec(vec) is iso and iso.isFailure()
    err = capsys.readouterr().err
    assert "Input object is NULL." in err and "Input object is not volume dat." in err
    assert "Input object is not scalar field dat." in err
