"""The CUDA path (C ABI, both kernel families) against the golden fixtures
made from the reference build, bit for bit."""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300.marching_cubes import MarchingCubes, PolygonObject, StructuredVolumeObject, TransferFunction

from .helpers import first_diff, golden, golden_inputs, golden_outputs, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", [_abi.PATH_AUTO, _abi.PATH_GATHER], ids=["auto", "gather"])
def test_cuda_matches_golden(kvsmc_ctx, path):
    man, arr = golden()
    kvsmc_ctx.set_kernel_path(path)
    try:
        for e in man:
            v, rect = golden_inputs(e, arr)
            g = golden_outputs(e, arr)
            vol = StructuredVolumeObject(v)
            if rect is not None:
                vol.setGridTypeToRectilinear()
                vol.setCoords(rect)
            if e["minmax"]:
                vol.setMinMaxValues(*e["minmax"])
            if e["obj"]:
                vol.setMinMaxObjectCoords(*e["obj"])
            tf = TransferFunction(256)
            if e["tf_range"]:
                tf.setRange(*e["tf_range"])
            nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
            mc = MarchingCubes(vol, e["iso"], nt, e["duplication"], tf, context=kvsmc_ctx)
            tag = e["key"]
            assert mc.isSuccess() == e["success"], tag
            assert same_bits(mc.coords(), g["coords"]), (tag, first_diff(mc.coords(), g["coords"]))
            assert same_bits(mc.normals(), g["normals"]), (tag, first_diff(mc.normals(), g["normals"]))
            assert np.array_equal(mc.connections(), g["connections"]), tag
            if np.isfinite(e["vol_min"]) or not g["coords"].size:
                assert np.array_equal(mc.colors(), g["colors"]), tag
            assert mc.polygonType() == e["polygon_type"] and mc.colorType() == e["color_type"], tag
            assert mc.normalType() == e["normal_type_out"], tag
    finally:
        kvsmc_ctx.set_kernel_path(_abi.PATH_AUTO)
