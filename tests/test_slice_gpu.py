"""kvs_gb300.slice_plane.SlicePlane (kvs::SlicePlane on the GPU) against the
fixtures made from the reference SlicePlane, bit for bit: coordinates,
per-vertex colours, normals (signed zeros included), types and bounding box,
for all ten value types, both constructor forms, planes through nodes and
planes that miss the volume."""
import ctypes as C

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300.marching_cubes import PolygonObject, StructuredVolumeObject, TransferFunction
from kvs_gb300.slice_plane import SlicePlane

from .helpers import first_diff, same_bits
from .test_slice_cpu import slice_fixtures

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run(e, v, ctx):
    tf = TransferFunction(256)
    if e["tf_range"]:
        tf.setRange(*e["tf_range"])
    vol = StructuredVolumeObject(v)
    if e["coefficients"] is not None:
        return SlicePlane(vol, coefficients=e["coefficients"], transfer_function=tf, context=ctx)
    return SlicePlane(vol, point=e["point"], normal=e["normal"], transfer_function=tf, context=ctx)


def test_slice_matches_reference_fixtures(kvsmc_ctx):
    man, arr = slice_fixtures()
    for e in man:
        k = e["key"]
        s = _run(e, arr[f"{e['case']}__input"], kvsmc_ctx)
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


def test_device_outputs_and_capacity(kvsmc_ctx):
    man, arr = slice_fixtures()
    e = next(x for x in man if x["key"] == "blob_f32__0")
    v = arr[f"{e['case']}__input"]
    host = _run(e, v, kvsmc_ctx)
    dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    table = np.ascontiguousarray(TransferFunction(256).table, np.uint8)
    p = _abi.SliceParams()
    coef = host.coefficients()
    for i in range(4):
        p.coefficients[i] = float(coef[i])
    for i in range(3):
        p.min_coord[i] = 0.0
        p.scale[i] = 1.0
    p.tf_min, p.tf_max = float(v.min()), float(v.max())
    p.tf_resolution, p.tf_table = 256, table.ctypes.data
    n = C.c_uint64(0)
    kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_slice_count(kvsmc_ctx.handle, dv.handle, C.byref(p), C.byref(n)), "count")
    assert n.value == e["ntriangles"]
    t = n.value
    c = torch.full((9 * t + 9,), -7.0, dtype=torch.float32, device="cuda")
    k = torch.zeros(9 * t + 9, dtype=torch.uint8, device="cuda")
    nn = torch.full((3 * t + 3,), -7.0, dtype=torch.float32, device="cuda")
    st = kvsmc_ctx.lib.kvsmc_slice_extract_device(kvsmc_ctx.handle, dv.handle, C.byref(p), c.data_ptr(), 9 * t - 9,
                                                  k.data_ptr(), 9 * t, nn.data_ptr(), 3 * t, C.byref(n))
    assert st == _abi.ERR_CAPACITY and n.value == t
    assert torch.all(c == -7.0)
    kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_slice_extract_device(kvsmc_ctx.handle, dv.handle, C.byref(p), c.data_ptr(),
                                                             9 * t, k.data_ptr(), 9 * t, nn.data_ptr(), 3 * t,
                                                             C.byref(n)), "extract")
    assert same_bits(c[:9 * t].cpu().numpy(), host.coords())       # the host call's min_coord 0, scale 1
    assert np.array_equal(k[:9 * t].cpu().numpy(), host.colors())
    assert same_bits(nn[:3 * t].cpu().numpy(), host.normals())
    assert float(c[9 * t]) == -7.0 and float(nn[3 * t]) == -7.0


def test_slice_rejects_like_the_reference(kvsmc_ctx, capsys):
    s = SlicePlane(coefficients=(0, 0, 1, -1), context=kvsmc_ctx)
    assert s.exec(None) is None and s.isFailure()
    assert s.exec(np.zeros(3)) is None
    vec = StructuredVolumeObject(np.zeros(4 * 4 * 4 * 3, np.float32), resolution=(4, 4, 4), veclen=3)
    assert s.exec(vec) is s
    err = capsys.readouterr().err
    assert "Input object is NULL." in err and "Input object is not volume dat." in err
    assert "Input volume is not a sclar field data." in err


def test_large_volumes_match_oracle(kvsmc_ctx):
    """The CUDA slicer against the restatement (oracle/slice.py) on volumes
    with long rows and planes that cut long runs of cells per row."""
    from oracle import slice as OS
    from .helpers import golden
    from .test_slice_cpu import default_tf_range, large_slice_cases
    table = golden()[1]["colormap256"]
    for name, v, coef in large_slice_cases():
        s = SlicePlane(StructuredVolumeObject(v), coefficients=coef, transfer_function=TransferFunction(256),
                       context=kvsmc_ctx)
        lo, hi = default_tf_range(v)
        c, rgb, n = OS.slice_plane(v, coef, table, lo, hi)
        assert c.size > 0, name
        assert same_bits(s.coords(), c), (name, first_diff(s.coords(), c))
        assert np.array_equal(s.colors(), rgb), name
        assert same_bits(s.normals(), n), name
