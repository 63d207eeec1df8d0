"""Host decisions of the Python mirror (kvs_gb300/marching_cubes.py) that run
without a GPU, against the reference's outputs in the golden fixtures: the
object colour (ColorMap::at, ColorMap.cpp:1043-1054) and the default
transfer function's table."""
import numpy as np

from kvs_gb300.marching_cubes import TransferFunction

from .helpers import golden, same_bits


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


def test_cells_mapper_host_decisions_match_reference(monkeypatch):
    """The unstructured mappers' host side (e.g. MarchingTetrahedra.cpp:94-136)
    on every cells fixture, with the device calls replaced: the extraction by
    the fixture's outputs and min/max, the bounding-box fold by its numpy
    restatement.  Success flag, types, the volume's min/max cache, colour,
    opacity and bounding box as the reference reported them."""
    from kvs_gb300 import _abi
    from kvs_gb300 import marching_cells as mcells
    from kvs_gb300.marching_cubes import PolygonObject
    from oracle import cells as ocells

    from .test_cells_cpu import case_inputs, cells_fixtures
    man, arr = cells_fixtures()
    for e in man:
        k = e["key"]
        v, xyz, conn = case_inputs(arr, e)
        want_mm = arr[f"{k}__vol_minmax"]

        def fake_extract(ctx, ct, values, coords, connections, iso, minmax=None, k=k, want_mm=want_mm):
            sizes = dict(ntriangles=arr[f"{k}__coords"].size // 9, min_value=float(want_mm[0]),
                         max_value=float(want_mm[1]))
            return arr[f"{k}__coords"], arr[f"{k}__normals"], sizes

        def fake_bounds(ctx, ct, coords, connections):
            return ocells.min_max_coords(coords, connections)

        monkeypatch.setattr(_abi, "marching_cells_host", fake_extract)
        monkeypatch.setattr(_abi, "cells_bounds", fake_bounds)
        vol = mcells.UnstructuredVolumeObject(mcells.MAPPERS_BY_ABI[e["cell_type"]].CELL, v.size, conn.shape[0], 1,
                                              xyz, conn, v)
        if e["minmax"] is not None:
            vol.setMinMaxValues(*e["minmax"])
        tf = TransferFunction(256)
        if e["tf_range"]:
            tf.setRange(*e["tf_range"])
        nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
        if e["form"] == 1:
            continue   # the Isosurface form routes through the same mapper; its GPU test covers it
        m = mcells.MAPPERS_BY_ABI[e["cell_type"]](vol, e["iso"], nt, e["duplication"], tf, context=object())
        assert m.isSuccess() == e["success"], k
        assert np.array_equal(m.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(m.opacities(), arr[f"{k}__opacities"]), k
        assert (m.polygonType(), m.colorType(), m.normalType()) == (
            e["polygon_type"], e["color_type"], e["normal_type_out"]), k
        assert vol.hasMinMaxValues() == e["vol_has_minmax"], k
        assert np.array_equal(m.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(m.maxObjectCoord(), np.float32(e["max_obj"])), k
        assert np.array_equal(m.maxExternalCoord(), np.float32(e["max_ext"])), k


def test_isosurface_host_decisions_match_reference(monkeypatch, oracle_lib):
    """kvs::Isosurface's structured branch (Isosurface.cpp:23-191) through the
    mirror on every isosurface fixture, with the device calls replaced: the
    min/max scan by the oracle's GetMinMaxValues restatement, the extraction
    by the fixture's outputs.  The isolevel and mode it hands to the device,
    then success flag, types, colour, bounding box and the volume's min/max
    cache as the reference reported them."""
    from kvs_gb300 import _abi
    from kvs_gb300 import marching_cubes as M
    from kvs_gb300.isosurface import Isosurface

    from .test_isosurface_cpu import effective, fixtures
    man, arr = fixtures()
    for e in man:
        k = e["key"]
        v = arr[f"{e['case']}__input"]
        iso_want, dup_want = effective(e, v, oracle_lib.minmax)
        mode_want = (_abi.MODE_SHARED_VERTEX_NORMAL if e["normal_type"] == "vertex"
                     else _abi.MODE_DUP_POLYGON_NORMAL if dup_want else _abi.MODE_SHARED_POLYGON_NORMAL)

        class FakeVolume:
            def __init__(self, values):
                self.values = values

            @classmethod
            def upload(cls, ctx, values):
                return cls(values)

            def minmax(self):
                return oracle_lib.minmax(self.values)

            def free(self):
                pass

        def fake(ctx, values, params, e=e, k=k, iso_want=iso_want, mode_want=mode_want):
            assert params.isolevel == iso_want and params.mode == mode_want, k
            return (arr[f"{k}__coords"], arr[f"{k}__normals"], arr[f"{k}__connections"],
                    dict(min_value=e["vol_min"], max_value=e["vol_max"],
                         extracted=not M._equal(e["vol_min"], e["vol_max"])))

        monkeypatch.setattr(_abi, "DeviceVolume", FakeVolume)
        monkeypatch.setattr(_abi, "marching_cubes_host", fake)
        vol = M.StructuredVolumeObject(v)
        if e["minmax"]:
            vol.setMinMaxValues(*e["minmax"])
        nt = M.PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else M.PolygonObject.VertexNormal
        ctx = object()
        if e["form"] == 0:
            iso = Isosurface(vol, normal_type=nt, context=ctx)
        elif e["form"] == 1:
            iso = Isosurface(vol, e["isolevel"], nt, context=ctx)
        else:
            tf = TransferFunction(256)
            if e["tf_range"]:
                tf.setRange(*e["tf_range"])
            iso = Isosurface(vol, e["isolevel"], nt, e["duplication"], tf, context=ctx)
        assert iso.isSuccess() == e["success"], k
        assert np.array_equal(iso.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(iso.opacities(), arr[f"{k}__opacities"]), k
        assert (iso.polygonType(), iso.normalType(), iso.colorType()) == (
            e["polygon_type"], e["normal_type_out"], e["color_type"]), k
        assert np.array_equal(iso.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(iso.maxExternalCoord(), np.float32(e["max_ext"])), k
        assert same_bits(np.float64([vol.minValue(), vol.maxValue()]), np.float64([e["vol_min"], e["vol_max"]])), k


def test_slice_plane_host_decisions_match_reference(monkeypatch, oracle_lib):
    """SlicePlane on structured volumes through the mirror (SlicePlane.cpp:
    setPlane, mapping) on every slice fixture, with the device calls replaced
    by the oracle (GetMinMaxValues restatement, oracle/slice.py for the
    extraction) fed with exactly the parameters the mirror hands to the
    device: the plane's coefficients, bounding box, scale and the transfer
    function's range.  Coordinates, colours and normals equal the
    reference's bit for bit, and so do the types and bounding box."""
    from kvs_gb300 import _abi
    from kvs_gb300 import slice_plane as SP
    from kvs_gb300.marching_cubes import StructuredVolumeObject
    from oracle import slice as OS

    from .test_slice_cpu import slice_fixtures
    table = golden()[1]["colormap256"]
    man, arr = slice_fixtures()

    class FakeVolume:
        def __init__(self, values):
            self.values = values

        @classmethod
        def upload(cls, ctx, values):
            return cls(values)

        def minmax(self):
            return oracle_lib.minmax(self.values)

        def free(self):
            pass

    def fake_slice(ctx, dv, p):
        nz, ny, nx = dv.values.shape
        assert list(p.min_coord) == [0.0, 0.0, 0.0] and list(p.scale) == [1.0, 1.0, 1.0]
        c, rgb, n = OS.slice_plane(dv.values, np.float32(list(p.coefficients)), table, np.float32(p.tf_min),
                                   np.float32(p.tf_max))
        return c, n, rgb, c.size // 9

    monkeypatch.setattr(_abi, "DeviceVolume", FakeVolume)
    monkeypatch.setattr(SP, "slice_plane_host", fake_slice)
    for e in man:
        k = e["key"]
        v = arr[f"{e['case']}__input"]
        tf = TransferFunction(256)
        if e["tf_range"]:
            tf.setRange(*e["tf_range"])
        vol = StructuredVolumeObject(v)
        if e["coefficients"] is not None:
            s = SP.SlicePlane(vol, coefficients=e["coefficients"], transfer_function=tf, context=object())
        else:
            s = SP.SlicePlane(vol, point=e["point"], normal=e["normal"], transfer_function=tf, context=object())
        assert s.isSuccess() == e["success"], k
        assert same_bits(s.coords(), arr[f"{k}__coords"]), k
        assert same_bits(s.normals(), arr[f"{k}__normals"]), k
        assert np.array_equal(s.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(s.opacities(), arr[f"{k}__opacities"]), k
        assert (s.polygonType(), s.colorType(), s.normalType()) == (
            e["polygon_type"], e["color_type"], e["normal_type"]), k
        assert np.array_equal(s.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(s.maxExternalCoord(), np.float32(e["max_ext"])), k


def test_mapper_parameters_reproduce_reference(monkeypatch, oracle_lib):
    """The parameters the MarchingCubes mirror hands to the device (mode,
    isolevel, preset range, min_coord and scale as MarchingCubes.cpp:166-168
    decides them from the bounding box) fed to the oracle's extraction in
    place of the device reproduce the reference's arrays bit for bit on every
    golden case (uniform, rectilinear and preset object coordinates)."""
    from kvs_gb300 import _abi
    from kvs_gb300 import marching_cubes as M

    from .helpers import golden_inputs, golden_outputs
    man, arr = golden()
    cmap = arr["colormap256"]

    def fake(ctx, values, params):
        vmin, vmax = ((params.min_value, params.max_value) if params.has_minmax else oracle_lib.minmax(values))
        sizes = dict(min_value=vmin, max_value=vmax, extracted=not M._equal(vmin, vmax))
        if not sizes["extracted"]:
            z = np.zeros(0, np.float32)
            return z, z, np.zeros(0, np.uint32), sizes
        o = oracle_lib.extract(values, params.isolevel, params.mode, vmin, vmax, list(params.min_coord),
                               list(params.scale))
        return o["coords"], o["normals"], o["connections"], sizes

    monkeypatch.setattr(_abi, "marching_cubes_host", fake)
    for e in man:
        v, rect = golden_inputs(e, arr)
        g = golden_outputs(e, arr)
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
        k = e["key"]
        assert same_bits(m.coords(), g["coords"]), k
        assert same_bits(m.normals(), g["normals"]), k
        assert np.array_equal(m.connections(), g["connections"]), k
        if g["coords"].size:
            assert np.array_equal(m.colors(), g["colors"]), k
