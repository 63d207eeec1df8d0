"""CPU restatement of the reference's binary STL and PLY export of a triangle mesh.

Test infrastructure only (the checker for kvsmc_stl_records / kvsmc_write_stl
and kvsmc_ply_records / kvsmc_write_ply; imported by tests/ only).
Follows:
  PolygonExporter<kvs::Stl>::exec   Source/Core/Visualization/Exporter/PolygonExporter.cpp:78-176
    - no connections: the coords as they are; else coords expanded through the
      connections (:101-125);
    - VertexNormal: per triangle (normal0 + normal1 + normal2) / 3.0f in float,
      left to right (:127-147); PolygonNormal: the normals as they are (:149-152);
      any other normal type: no normals, so zero triangles are written;
  Stl::write_binary                 Source/Core/FileFormat/STL/Stl.cpp:490-540
    - 80 header bytes "Generated by KVS" zero-padded, uint32 count =
      normals.size() / 3 (wrapping like static_cast<UInt32>), then per triangle
      3 normal floats, 9 coordinate floats, 2 zero bytes.
"""
import numpy as np

VERTEX_NORMAL, POLYGON_NORMAL = 0, 1

RECORD = np.dtype([("n", "<f4", (3,)), ("c", "<f4", (9,)), ("attr", "<u2")])
assert RECORD.itemsize == 50


def stl_binary(coords, normals, connections, normal_type):
    coords = np.asarray(coords, np.float32).reshape(-1)
    normals = np.asarray(normals, np.float32).reshape(-1)
    conn = np.asarray(connections, np.uint32).reshape(-1)
    if conn.size == 0:
        c = coords.reshape(-1, 9) if coords.size else np.zeros((0, 9), np.float32)
    else:
        c = coords.reshape(-1, 3)[conn.reshape(-1, 3)].reshape(-1, 9)
    if normal_type == VERTEX_NORMAL:
        t = conn.reshape(-1, 3)
        nv = normals.reshape(-1, 3)
        s = (nv[t[:, 0]] + nv[t[:, 1]]) + nv[t[:, 2]]          # float32 adds, in order
        n = (s / np.float32(3.0)).astype(np.float32)
    elif normal_type == POLYGON_NORMAL:
        n = normals.reshape(-1, 3)
    else:
        n = np.zeros((0, 3), np.float32)
    count = n.shape[0]
    header = bytearray(84)
    header[:16] = b"Generated by KVS"
    header[80:84] = np.uint32(count & 0xFFFFFFFF).tobytes()
    rec = np.zeros(count, RECORD)
    rec["n"] = n
    rec["c"] = c[:count]
    return bytes(header) + rec.tobytes()


def ply_binary(coords, colors, normals, color_type="polygon", normal_type="polygon"):
    """PolygonExporter<kvs::Ply>::exec (PolygonExporter.cpp:178-361) + Ply::write
    (Ply.cpp:389-488, binary little endian; header PlyFile.cpp:399-460) of a
    triangle mesh without connections, as bytes: vertex colours = the single
    colour repeated (3 colour bytes) or the vertex colours (VertexColor);
    normals = zeros for PolygonNormal (averaged over connections, none here),
    the vertex normals for VertexNormal; 'element face 0' (faces are counted
    only from connections)."""
    c = np.asarray(coords, np.float32).reshape(-1, 3)
    k = np.asarray(colors, np.uint8).reshape(-1)
    n = np.asarray(normals, np.float32).reshape(-1)
    nv = c.shape[0]
    has_c, has_n = k.size > 0, n.size > 0
    head = "ply\nformat binary_little_endian 1.0\nelement vertex %d\n" % nv
    head += "property float x\nproperty float y\nproperty float z\n"
    if has_c:
        head += "property uchar red\nproperty uchar green\nproperty uchar blue\n"
    if has_n:
        head += "property float nx\nproperty float ny\nproperty float nz\n"
    head += "element face 0\nend_header\n"
    fields = [("xyz", "<f4", (3,))]
    if has_c:
        fields.append(("rgb", "u1", (3,)))
    if has_n:
        fields.append(("n", "<f4", (3,)))
    rec = np.zeros(nv, np.dtype(fields))
    rec["xyz"] = c
    if has_c:
        rec["rgb"] = np.broadcast_to(k[:3], (nv, 3)) if k.size == 3 else k.reshape(-1, 3)[:nv]
    if has_n:
        rec["n"] = n.reshape(-1, 3)[:nv] if normal_type == "vertex" else 0.0
    return head.encode() + rec.tobytes()
