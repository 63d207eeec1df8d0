"""ASCII STL (text formatted on the GPU) and KVSML polygon files against the
files the reference's own writers made (tests/golden/exports.npz), byte for
byte: through the Python mirrors of PolygonExporter<kvs::Stl> (ASCII, the
kvs::Stl default) and PolygonExporter<kvs::KVSMLPolygonObject> (each writing
data type), and from device meshes without a host PolygonObject.  The "%f"
formatter is also checked on random and edge-case floats against the C
library's conversion (Python's '%f' is correctly rounded, ties to even, the
same; NaN takes the C library's sign)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300.export import (PolygonExporterKVSML, PolygonExporterStl, write_kvsml_device,
                              write_stl_ascii_device)
from kvs_gb300.marching_cubes import MarchingCubes, PolygonObject, StructuredVolumeObject, TransferFunction
from oracle import export as E

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
MAN = json.load(open(os.path.join(HERE, "golden", "exports.json")))
ARR = np.load(os.path.join(HERE, "golden", "exports.npz"))


def _mc(e, ctx):
    nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
    return MarchingCubes(StructuredVolumeObject(ARR[f"{e['case']}__input"]), e["isolevel"], nt, e["duplication"],
                         TransferFunction(256), context=ctx)


@pytest.mark.parametrize("e", MAN, ids=[e["case"] for e in MAN])
def test_ascii_stl_matches_reference_file(kvsmc_ctx, tmp_path, e):
    ex = PolygonExporterStl(_mc(e, kvsmc_ctx), context=kvsmc_ctx)   # the default file type: ASCII
    p = tmp_path / "out.stl"
    assert ex.write(str(p))
    (fn,) = e["files"]["stl_ascii"]
    assert p.read_bytes() == ARR[f"{e['case']}__stl_ascii__{fn}"].tobytes()


@pytest.mark.parametrize("e", MAN, ids=[e["case"] for e in MAN])
def test_kvsml_matches_reference_files(kvsmc_ctx, tmp_path, e):
    mc = _mc(e, kvsmc_ctx)
    for fmt, setter in (("kvsml_ascii", "setWritingDataTypeToAscii"),
                        ("kvsml_external_ascii", "setWritingDataTypeToExternalAscii"),
                        ("kvsml_external_binary", "setWritingDataTypeToExternalBinary")):
        d = tmp_path / fmt
        d.mkdir()
        ex = PolygonExporterKVSML(mc, context=kvsmc_ctx)
        getattr(ex, setter)()
        assert ex.write(str(d / (e["case"] + ".kvsml")))
        assert sorted(os.listdir(d)) == e["files"][fmt], fmt
        for fn in e["files"][fmt]:
            assert (d / fn).read_bytes() == ARR[f"{e['case']}__{fmt}__{fn}"].tobytes(), (fmt, fn)


def _floats(rng, n):
    """Random floats over every exponent, plus values on six-decimal ties and edge cases."""
    bits = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32).copy()
    k = rng.integers(-2 ** 20, 2 ** 20, n // 4)
    ties = ((2 * k + 1).astype(np.float64) / 128.0).astype(np.float32)        # odd multiples of 2^-7: ties
    small = rng.standard_normal(n // 4).astype(np.float32) * np.float32(1e-6)
    mid = rng.uniform(-2000, 2000, n // 4).astype(np.float32)
    edges = np.array([0.0, -0.0, 0.5e-6, -0.5e-6, 4.9999e-7, 5.0001e-7, 0.9999995, 1.0 - 2 ** -24, 999999.5,
                      2 ** 63, 2 ** 64, 3.4028235e38, -3.4028235e38, 1e-45, -1e-45, np.inf, -np.inf, np.nan,
                      -np.nan, 0.0078125, 0.0234375, 1.5e-6, 2.5e-6], np.float32)
    return np.concatenate([x, ties, small, mid, edges])


@pytest.mark.parametrize("mode", [0, 2])
def test_fixed6_formatting_against_c_conversion(kvsmc_ctx, tmp_path, mode):
    rng = np.random.default_rng(17 + mode)
    v = _floats(rng, 80_000)
    ntri = v.size // 12
    v = v[:12 * ntri]
    if mode == _abi.MODE_DUP_POLYGON_NORMAL:
        normals, coords, conn = v[:3 * ntri], v[3 * ntri:], np.zeros(0, np.uint32)
    else:
        # shared vertices with vertex normals: the normal written is (n0 + n1 + n2) / 3
        coords, normals = v[:6 * ntri], v[6 * ntri:12 * ntri]
        conn = rng.integers(0, 2 * ntri, 3 * ntri).astype(np.uint32)
    p = tmp_path / "f.stl"
    st = kvsmc_ctx.lib.kvsmc_write_stl_ascii_host(kvsmc_ctx.handle, str(p).encode(), mode, coords.ctypes.data,
                                                  coords.size, normals.ctypes.data, normals.size,
                                                  conn.ctypes.data if conn.size else None, conn.size)
    assert st == _abi.OK, _abi.status_string(st)
    want = E.stl_ascii(coords, normals, conn, E.POLYGON_NORMAL if mode == 0 else E.VERTEX_NORMAL)
    got = p.read_bytes()
    if mode != _abi.MODE_DUP_POLYGON_NORMAL:
        # normals averaged from NaN inputs: the sign of a NaN that arithmetic
        # produces is not specified (x86, Arm and the GPU differ)
        got, want = got.replace(b"-nan", b"nan"), want.replace(b"-nan", b"nan")
    if got != want:
        a, b = got.split(b"\n"), want.split(b"\n")
        i = next(i for i in range(min(len(a), len(b))) if a[i] != b[i])
        raise AssertionError((i, a[i], b[i]))


def test_chunks_and_device_meshes(kvsmc_ctx, tmp_path):
    """More than one 2^20-triangle chunk, from device arrays; and a device mesh
    to KVSML without a host polygon object."""
    rng = np.random.default_rng(5)
    ntri = (1 << 20) + 4099
    coords = (rng.standard_normal(9 * ntri) * 300).astype(np.float32)
    normals = rng.standard_normal(3 * ntri).astype(np.float32)
    c = torch.from_numpy(coords).cuda()
    n = torch.from_numpy(normals).cuda()
    p = tmp_path / "big.stl"
    write_stl_ascii_device(kvsmc_ctx, p, 0, c.data_ptr(), n.data_ptr(), None, 3 * ntri, ntri)
    assert p.read_bytes() == E.stl_ascii(coords, normals, np.zeros(0, np.uint32), E.POLYGON_NORMAL)
    small = 5000
    q = tmp_path / "m.kvsml"
    write_kvsml_device(kvsmc_ctx, q, 2, 0, c.data_ptr(), 9 * small, n.data_ptr(), 3 * small, None, 0,
                       np.array([1, 2, 3], np.uint8), np.array([255], np.uint8))
    want = E.kvsml_polygon("m", 2, coords[:9 * small], normals[:3 * small], np.zeros(0, np.uint32), "polygon",
                           [1, 2, 3], [255])
    for fn, data in want.items():
        assert (tmp_path / fn).read_bytes() == data, fn
