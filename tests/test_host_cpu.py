"""Host decisions of the Python mirror (kvs_gb300/marching_cubes.py) that run
without a GPU, against the reference's outputs in the golden fixtures: the
object colour (ColorMap::at, ColorMap.cpp:1043-1054) and the default
transfer function's table."""
import numpy as np

from kvs_gb300.marching_cubes import TransferFunction

from .helpers import golden


def test_default_table_is_the_references():
    _, arr = golden()
    assert np.array_equal(TransferFunction().table, arr["colormap256"].reshape(256, 3))


def test_color_at_matches_reference():
    _, arr = golden()
    tf = TransferFunction(256, arr["colormap256"])
    tf.setRange(-1.0, 2.0)
    assert tf.hasRange()
    for v, want in zip(arr["color_at_values"], arr["color_at_rgb"]):
        assert np.array_equal(tf.color_at(float(v)), want), (v, tf.color_at(float(v)), want)


def test_range_rules():
    tf = TransferFunction()
    assert not tf.hasRange()
    tf.setRange(0.5, 0.5 + 1e-7)   # kvs::Math::Equal: closer than 1e-6 is no range
    assert not tf.hasRange()
    c = tf.copy()
    c.setRange(0.0, 1.0)
    assert c.hasRange() and not tf.hasRange()


def test_bounding_box_matches_reference():
    """MapperBase::setMinMaxCoords through the mirror's
    StructuredVolumeObject.updateMinMaxCoords (uniform and rectilinear grids,
    preset object coordinates) for every golden case."""
    from kvs_gb300.marching_cubes import StructuredVolumeObject

    from .helpers import golden_inputs
    man, arr = golden()
    n = 0
    for e in man:
        v, rect = golden_inputs(e, arr)
        nz, ny, nx = v.shape
        vol = StructuredVolumeObject(values=v.ravel(), resolution=(nx, ny, nz))
        if rect is not None:
            vol.setGridTypeToRectilinear()
            vol.setCoords(np.asarray(rect, np.float32))
        if e["obj"]:
            vol.setMinMaxObjectCoords(e["obj"][0], e["obj"][1])
        if not vol.hasMinMaxObjectCoords():
            vol.updateMinMaxCoords()
        assert np.array_equal(vol.minObjectCoord(), np.array(e["min_obj"], np.float32)), e["key"]
        assert np.array_equal(vol.maxObjectCoord(), np.array(e["max_obj"], np.float32)), e["key"]
        n += 1
    assert n > 800


def test_object_colour_matches_reference():
    """MapperBase::setRange's transfer-function range (MapperBase.cpp:54-83:
    int8 and uint8 fixed ranges, else the volume's min/max, widened by 1 when
    they are equal) and the colour at the isolevel, for every golden case with
    a surface."""
    from kvs_gb300 import _abi
    from kvs_gb300.marching_cubes import set_mapper_range

    from .helpers import golden_inputs, golden_outputs
    man, arr = golden()
    n = 0
    for e in man:
        v, _ = golden_inputs(e, arr)
        g = golden_outputs(e, arr)
        if not g["coords"].size or not np.isfinite(e["vol_min"]):
            continue
        tf = TransferFunction(256, arr["colormap256"])
        if e["tf_range"]:
            tf.setRange(*e["tf_range"])
        set_mapper_range(tf, _abi.dtype_code(v.dtype), e["vol_min"], e["vol_max"])
        assert np.array_equal(tf.color_at(e["iso"]), g["colors"]), e["key"]
        n += 1
    assert n > 500


def test_mapper_host_decisions_match_reference(monkeypatch):
    """MarchingCubes.exec/mapping's host side (MarchingCubes.cpp:46-132) on
    every golden case, with the device call replaced by the case's fixture
    outputs: the mode and preset range it asks for, then the success flag,
    polygon / normal / colour types, colour, opacity and bounding box it
    reports."""
    from kvs_gb300 import _abi
    from kvs_gb300 import marching_cubes as M

    from .helpers import golden_inputs, golden_outputs
    man, arr = golden()
    cmap = arr["colormap256"]
    for e in man:
        v, rect = golden_inputs(e, arr)
        g = golden_outputs(e, arr)
        want_mode = (_abi.MODE_SHARED_VERTEX_NORMAL if e["normal_type"] == "vertex"
                     else _abi.MODE_DUP_POLYGON_NORMAL if e["duplication"] else _abi.MODE_SHARED_POLYGON_NORMAL)

        def fake(ctx, values, params, e=e, g=g, want_mode=want_mode):
            assert params.mode == want_mode and params.isolevel == e["iso"], e["key"]
            assert params.has_minmax == (1 if e["minmax"] else 0), e["key"]
            extracted = not M._equal(e["vol_min"], e["vol_max"])
            sizes = dict(ntriangles=e["ntriangles"], min_value=e["vol_min"], max_value=e["vol_max"],
                         extracted=extracted)
            return g["coords"], g["normals"], g["connections"], sizes

        monkeypatch.setattr(_abi, "marching_cubes_host", fake)
        nz, ny, nx = v.shape
        vol = M.StructuredVolumeObject(values=v.ravel(), resolution=(nx, ny, nz))
        if rect is not None:
            vol.setGridTypeToRectilinear()
            vol.setCoords(np.asarray(rect, np.float32))
        if e["obj"]:
            vol.setMinMaxObjectCoords(e["obj"][0], e["obj"][1])
        if e["minmax"]:
            vol.setMinMaxValues(*e["minmax"])
        tf = M.TransferFunction(256, cmap)
        if e["tf_range"]:
            tf.setRange(*e["tf_range"])
        nt = M.PolygonObject.VertexNormal if e["normal_type"] == "vertex" else M.PolygonObject.PolygonNormal
        m = M.MarchingCubes(vol, e["iso"], nt, e["duplication"], tf, context=object())
        tag = e["key"]
        assert m.isSuccess() == e["success"], tag
        assert m.polygonType() == e["polygon_type"], tag
        assert m.normalType() == e["normal_type_out"], tag
        assert m.colorType() == e["color_type"], tag
        assert np.array_equal(m.minObjectCoord(), np.array(e["min_obj"], np.float32)), tag
        assert np.array_equal(m.maxObjectCoord(), np.array(e["max_obj"], np.float32)), tag
        if g["coords"].size:
            assert np.array_equal(m.colors(), g["colors"]), tag
            assert np.array_equal(m.opacities(), [255]), tag
            assert m.coords() is g["coords"], tag
        else:
            assert m.coords().size == 0, tag
