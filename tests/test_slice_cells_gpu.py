"""kvs_gb300.slice_plane.SlicePlane on unstructured volumes
(kvsmc_slice_cells_host) against the fixtures made from the reference
SlicePlane, bit for bit (coordinates, per-vertex colours, normals, types,
bounding box, the volume's min/max cache), and against the numpy
restatement on grids of a million and more cells."""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import marching_cells as mcells
from kvs_gb300.marching_cubes import TransferFunction
from kvs_gb300.slice_plane import SlicePlane, slice_cells_host
from oracle import cells as ocells

from . import cell_meshes as cm
from .helpers import first_diff, golden, same_bits
from .test_slice_cells_cpu import case_inputs, plane_of, slice_cells_fixtures

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _volume(ct, v, xyz, conn):
    return mcells.UnstructuredVolumeObject(mcells.MAPPERS_BY_ABI[ct].CELL, v.size, conn.shape[0], 1, xyz, conn, v)


def test_slice_cells_matches_reference_fixtures(kvsmc_ctx):
    man, arr = slice_cells_fixtures()
    for e in man:
        k = e["key"]
        v, xyz, conn = case_inputs(arr, e)
        vol = _volume(e["cell_type"], v, xyz, conn)
        tf = TransferFunction(256)
        if e["tf_range"]:
            tf.setRange(*e["tf_range"])
        if e["coefficients"] is not None:
            s = SlicePlane(vol, coefficients=e["coefficients"], transfer_function=tf, context=kvsmc_ctx)
        else:
            s = SlicePlane(vol, point=e["point"], normal=e["normal"], transfer_function=tf, context=kvsmc_ctx)
        assert s.isSuccess() == e["success"], k
        for f, got in (("coords", s.coords()), ("normals", s.normals())):
            want = arr[f"{k}__{f}"]
            assert same_bits(got, want), (k, f, first_diff(got, want))
        assert np.array_equal(s.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(s.opacities(), arr[f"{k}__opacities"]), k
        assert (s.polygonType(), s.colorType(), s.normalType()) == (
            e["polygon_type"], e["color_type"], e["normal_type"]), k
        assert np.array_equal(s.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(s.maxExternalCoord(), np.float32(e["max_ext"])), k
        if conn.size:
            assert same_bits(np.array([vol.minValue(), vol.maxValue()]), arr[f"{k}__vol_minmax"]), k


@pytest.mark.parametrize("ct", [0, 1, 2, 3])
def test_large_grids_match_oracle(kvsmc_ctx, ct):
    xyz, conn = cm.grid(ct, 64, 64, 64, jitter=0.3, seed=60 + ct)
    v = cm.sphere_values(xyz, (30.3, 31.7, 29.1))
    table = golden()[1]["colormap256"]
    for coef in ((0.31, -0.52, 0.79, -10.0), (0.0, 0.0, 1.0, -31.0)):
        p = _abi.SliceParams()
        for i in range(4):
            p.coefficients[i] = float(np.float32(coef[i]))
        tbl = np.ascontiguousarray(table, np.uint8)
        p.tf_min, p.tf_max, p.tf_resolution, p.tf_table = 0.5, 40.0, 256, tbl.ctypes.data
        c, n, rgb, t = slice_cells_host(kvsmc_ctx, ct, v, xyz, conn, p)
        oc, orgb, on = ocells.slice_cells(ct, v, xyz, conn, np.float32(coef), table, np.float32(0.5), np.float32(40.0))
        assert t * 9 == oc.size > 0
        assert same_bits(c, oc), (ct, coef, first_diff(c, oc))
        assert np.array_equal(rgb, orgb) and same_bits(n, on), (ct, coef)


def test_bad_connection_index_is_an_error(kvsmc_ctx):
    xyz, conn = cm.grid(0, 6, 6, 6, seed=2)
    v = cm.sphere_values(xyz)
    bad = conn.copy()
    bad[5, 2] = 10 ** 6
    p = _abi.SliceParams()
    for i, c in enumerate((0.3, -0.5, 0.8, -1.0)):
        p.coefficients[i] = c
    tbl = np.ascontiguousarray(golden()[1]["colormap256"], np.uint8)
    p.tf_min, p.tf_max, p.tf_resolution, p.tf_table = 0.0, 5.0, 256, tbl.ctypes.data
    with pytest.raises(_abi.KvsmcError, match="connection index"):
        slice_cells_host(kvsmc_ctx, 0, v, xyz, bad, p)
