"""GPU binary STL serialisation (kvsmc_stl_records, kvsmc_write_stl,
kvsmc_write_stl_host) against files written by the reference exporter and
against the restatement in oracle/export.py, byte for byte."""
import ctypes as C

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300.export import PolygonExporterStl, stl_records_device, write_stl_device
from kvs_gb300.marching_cubes import MarchingCubes, PolygonObject, StructuredVolumeObject, TransferFunction
from oracle import export as E

from .test_export_cpu import stl_fixtures

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _mc(e, v, ctx):
    nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
    return MarchingCubes(StructuredVolumeObject(v), e["isolevel"], nt, e["duplication"], TransferFunction(256),
                         context=ctx)


def test_exporter_matches_reference_files(kvsmc_ctx, tmp_path):
    man, arr = stl_fixtures()
    for e in man:
        k = e["case"]
        mc = _mc(e, arr[f"{k}__input"], kvsmc_ctx)
        ex = PolygonExporterStl(mc, context=kvsmc_ctx)
        ex.setFileType("binary")
        p = tmp_path / f"{k}.stl"
        assert ex.write(str(p)), k
        assert p.read_bytes() == arr[f"{k}__stl"].tobytes(), k


def _device_mesh(ctx, e, v):
    """Extract on the device (kvsmc_extract_device); returns the torch buffers and sizes."""
    dv = _abi.DeviceVolume.upload(ctx, v)
    mode = (_abi.MODE_SHARED_VERTEX_NORMAL if e["normal_type"] == "vertex" else
            (_abi.MODE_DUP_POLYGON_NORMAL if e["duplication"] else _abi.MODE_SHARED_POLYGON_NORMAL))
    p = _abi.make_params(e["isolevel"], mode)
    s = _abi.Sizes()
    ctx.check(ctx.lib.kvsmc_count(ctx.handle, dv.handle, C.byref(p), C.byref(s)), "count")
    c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
    n = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
    k = torch.empty(max(1, s.nconnections), dtype=torch.int32, device="cuda")
    ctx.check(ctx.lib.kvsmc_extract_device(ctx.handle, dv.handle, C.byref(p), c.data_ptr(), s.ncoords,
                                           n.data_ptr(), s.nnormals, k.data_ptr(), s.nconnections, C.byref(s)),
              "extract")
    return mode, c, n, k, s


def test_device_mesh_to_file_without_host_polygon(kvsmc_ctx, tmp_path):
    man, arr = stl_fixtures()
    for e in man:
        key = e["case"]
        mode, c, n, k, s = _device_mesh(kvsmc_ctx, e, arr[f"{key}__input"])
        p = tmp_path / f"{key}.stl"
        write_stl_device(kvsmc_ctx, p, mode, c.data_ptr(), n.data_ptr(),
                         k.data_ptr() if mode else None, s.nvertices, s.ntriangles)
        want = arr[f"{key}__stl"].tobytes()
        assert p.read_bytes() == want, key
        if s.ntriangles:
            out = torch.empty(50 * s.ntriangles, dtype=torch.uint8, device="cuda")
            stl_records_device(kvsmc_ctx, mode, c.data_ptr(), n.data_ptr(), k.data_ptr() if mode else None,
                               s.nvertices, s.ntriangles, out.data_ptr())
            assert out.cpu().numpy().tobytes() == want[84:], key


@pytest.mark.parametrize("ntri", [1, 255, 256, 257, 3 * 256 + 17, (1 << 20) + 3])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_tiles_and_chunks_against_restatement(kvsmc_ctx, tmp_path, ntri, mode):
    rng = np.random.default_rng(ntri * 3 + mode)
    if mode == _abi.MODE_DUP_POLYGON_NORMAL:
        coords = rng.standard_normal(9 * ntri).astype(np.float32)
        conn = np.zeros(0, np.uint32)
        normals = rng.standard_normal(3 * ntri).astype(np.float32)
        nt = E.POLYGON_NORMAL
    else:
        nv = max(3, ntri // 2)
        coords = rng.standard_normal(3 * nv).astype(np.float32)
        conn = rng.integers(0, nv, 3 * ntri).astype(np.uint32)
        normals = rng.standard_normal(3 * (ntri if mode == 1 else nv)).astype(np.float32)
        nt = E.POLYGON_NORMAL if mode == 1 else E.VERTEX_NORMAL
    want = E.stl_binary(coords, normals, conn, nt)
    c = torch.from_numpy(coords).cuda()
    n = torch.from_numpy(normals).cuda()
    k = torch.from_numpy(conn.view(np.int32)).cuda() if conn.size else None
    p = tmp_path / "m.stl"
    write_stl_device(kvsmc_ctx, p, mode, c.data_ptr(), n.data_ptr(), k.data_ptr() if k is not None else None,
                     coords.size // 3, ntri)
    got = p.read_bytes()
    assert len(got) == len(want) and got == want


def test_bad_connection_index_is_refused(kvsmc_ctx, tmp_path):
    coords = torch.zeros(9, dtype=torch.float32, device="cuda")
    normals = torch.zeros(3, dtype=torch.float32, device="cuda")
    conn = torch.tensor([0, 1, 7], dtype=torch.int32, device="cuda")   # vertex 7 of 3
    out = torch.empty(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(_abi.KvsmcError):
        stl_records_device(kvsmc_ctx, 1, coords.data_ptr(), normals.data_ptr(), conn.data_ptr(), 3, 1,
                           out.data_ptr())
    with pytest.raises(_abi.KvsmcError):
        write_stl_device(kvsmc_ctx, tmp_path / "bad.stl", 2, coords.data_ptr(), normals.data_ptr(),
                         conn.data_ptr(), 3, 1)
    # the context still works afterwards
    good = torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda")
    stl_records_device(kvsmc_ctx, 1, coords.data_ptr(), normals.data_ptr(), good.data_ptr(), 3, 1, out.data_ptr())


def test_exporter_checks_like_the_reference(kvsmc_ctx, tmp_path, capsys):
    ex = PolygonExporterStl(context=kvsmc_ctx)
    assert ex.exec(None) is None and ex.isFailure()
    assert ex.exec(np.zeros(3)) is None
    err = capsys.readouterr().err
    assert "Input object is NULL." in err and "Input object is not polygon object." in err
    v = np.zeros((3, 3, 3), np.float32)
    v[1, 1, 1] = 1
    mc = MarchingCubes(StructuredVolumeObject(v), 0.5, context=kvsmc_ctx)
    ex = PolygonExporterStl(mc, context=kvsmc_ctx)
    assert ex.write(str(tmp_path / "a.stl"))              # ASCII, the default file type (Stl.cpp:86)
    assert (tmp_path / "a.stl").read_bytes().startswith(b"solid Generated by KVS\nfacet normal ")
    ex.setFileType("binary")
    assert ex.write(str(tmp_path / "b.stl"))


def test_ply_exporter_matches_reference_files(kvsmc_ctx, tmp_path):
    from kvs_gb300.export import PolygonExporterPly

    from .test_ply_cpu import ply_fixtures, polygon_of
    man, arr = ply_fixtures()
    for e in man:
        ex = PolygonExporterPly(polygon_of(arr, e), context=kvsmc_ctx)
        ex.setFileType("binary")
        p = tmp_path / f"{e['case']}.ply"
        assert ex.write(str(p)), e["case"]
        assert p.read_bytes() == arr[f"{e['case']}__file"].tobytes(), e["case"]


@pytest.mark.parametrize("nv", [1, 255, 256, 257, (1 << 21) + 300])
def test_ply_records_and_chunks_against_restatement(kvsmc_ctx, tmp_path, nv):
    """Record tiles (256 vertices), the last partial tile, and the 2^21-vertex
    file chunks, for every colour / normal mode."""
    from kvs_gb300.export import write_ply_device
    rng = np.random.default_rng(nv)
    c = torch.from_numpy(rng.standard_normal(3 * nv).astype(np.float32)).cuda()
    k = torch.from_numpy(rng.integers(0, 256, 3 * nv).astype(np.uint8)).cuda()
    n = torch.from_numpy(rng.standard_normal(3 * nv).astype(np.float32)).cuda()
    torch.cuda.synchronize()
    hc, hk, hn = c.cpu().numpy(), k.cpu().numpy(), n.cpu().numpy()
    for cm, nm in ((0, 0), (1, 1), (2, 1), (2, 2), (1, 0)):
        p = tmp_path / f"m{cm}{nm}.ply"
        write_ply_device(kvsmc_ctx, p, c.data_ptr(), nv, k.data_ptr(), cm, n.data_ptr(), nm)
        colors = hk[:3] if cm == 1 else (hk if cm == 2 else np.zeros(0, np.uint8))
        normals = hn if nm else np.zeros(0, np.float32)
        want = E.ply_binary(hc, colors, normals, "vertex" if cm == 2 else "polygon", "vertex" if nm == 2 else "polygon")
        assert p.read_bytes() == want, (nv, cm, nm)
        # the records alone, into device memory
        rec = kvsmc_ctx.lib.kvsmc_ply_record_bytes(cm, nm)
        out = torch.empty(nv * rec + 16, dtype=torch.uint8, device="cuda")
        kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_ply_records(kvsmc_ctx.handle, c.data_ptr(), nv, k.data_ptr(), cm,
                                                        n.data_ptr(), nm, out.data_ptr()), "ply_records")
        kvsmc_ctx.synchronize()
        hl = int(kvsmc_ctx.lib.kvsmc_ply_header(nv, cm, nm, None, 0))
        assert out[:nv * rec].cpu().numpy().tobytes() == want[hl:], (nv, cm, nm)
