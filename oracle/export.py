"""CPU restatement of the reference's binary STL export of a triangle mesh.

Test infrastructure only (the checker for kvsmc_stl_records / kvsmc_write_stl).
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
