"""CPU restatement of the reference's STL (binary and ASCII), KVSML polygon and
PLY export of a triangle mesh.

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


def _c_fixed6(x):
    """C's "%f" of a float promoted to double: Python's correctly rounded
    '%f' (ties to even, as the C library), with the C library's sign on NaN."""
    x = float(x)
    if x != x:
        return ("-" if np.signbit(x) else "") + "nan"
    return "%f" % x


def stl_ascii(coords, normals, connections, normal_type):
    """PolygonExporter<kvs::Stl>::exec (as stl_binary) + Stl::write_ascii
    (Stl.cpp:447-480) as bytes: "solid Generated by KVS", per triangle
    "facet normal %f %f %f", "outer loop", three "vertex %f %f %f", "endloop",
    "endfacet", then "endsolid"."""
    b = stl_binary(coords, normals, connections, normal_type)
    rec = np.frombuffer(b[84:], RECORD)
    out = ["solid Generated by KVS\n"]
    for r in rec:
        n, c = r["n"], r["c"]
        out.append("facet normal %s %s %s\nouter loop\n" % tuple(_c_fixed6(v) for v in n))
        for k in range(3):
            out.append("vertex %s %s %s\n" % tuple(_c_fixed6(v) for v in c[3 * k:3 * k + 3]))
        out.append("endloop\nendfacet\n")
    out.append("endsolid\n")
    return "".join(out).encode()


def _g6(v):
    """An ostream's default output of a float (six significant digits: "%g")."""
    v = float(v)
    if v != v:
        return ("-" if np.signbit(v) else "") + "nan"
    return "%.6g" % v


def kvsml_polygon(base, writing_type, coords, normals, connections, normal_type, color, opacity):
    """PolygonExporter<kvs::KVSMLPolygonObject>::exec (PolygonExporter.cpp:22-68)
    + KVSMLPolygonObject::write (KVSMLPolygonObject.cpp:349-492) of a triangle
    mesh with one polygon colour: {file name: bytes} of the .kvsml file (named
    base + ".kvsml") and its external data files.  writing_type 0 Ascii, 1
    ExternalAscii, 2 ExternalBinary (DataArrayTag.h:110-169, DataArray.h:365-440:
    internal values each followed by a blank, then a newline and the closing
    tag's indentation; external ASCII values each followed by ", "; binary the
    raw little-endian array).  normal_type "vertex" puts the normals under
    <Vertex>, "polygon" under <Polygon>."""
    coords = np.asarray(coords, np.float32).reshape(-1)
    normals = np.asarray(normals, np.float32).reshape(-1)
    conn = np.asarray(connections, np.uint32).reshape(-1)
    files = {}
    nv = coords.size // 3
    npoly = conn.size // 3 if conn.size else nv // 3
    x = ['<?xml version="1.0" ?>\n', "<!-- Generated by kvs::KVSMLPolygonObject::write() -->\n", "<KVSML>\n",
         '    <Object type="PolygonObject">\n',
         '        <PolygonObject polygon_type="triangle" color_type="polygon" normal_type="%s">\n' % normal_type]

    def array(ind, kind, a, is_float):
        t = "float" if is_float else "uint"
        fmt = _g6 if is_float else (lambda v: "%d" % v)
        if writing_type == 0:
            x.append('%s<DataArray type="%s">' % (ind, t) + "".join(fmt(v) + " " for v in a) + "\n%s</DataArray>\n" % ind)
            return
        fn = "%s_%s.dat" % (base, kind)
        x.append('%s<DataArray type="%s" format="%s" file="%s"%s />\n'
                 % (ind, t, "ascii" if writing_type == 1 else "binary", fn,
                    ' endian="little"' if writing_type == 2 else ""))
        files[fn] = ("".join(fmt(v) + ", " for v in a).encode() if writing_type == 1
                     else np.ascontiguousarray(a).astype("<f4" if is_float else "<u4").tobytes())

    def element(ind, tag, kind, a, is_float):
        if a.size == 0:
            return
        x.append("%s<%s>\n" % (ind, tag))
        array(ind + "    ", kind, a, is_float)
        x.append("%s</%s>\n" % (ind, tag))

    def value(ind, tag, v):
        if v is None or len(v) == 0:
            return
        x.append("%s<%s>\n%s    <DataValue>" % (ind, tag, ind) + "".join("%d " % int(e) for e in v)
                 + "\n%s    </DataValue>\n%s</%s>\n" % (ind, ind, tag))

    ind = " " * 16

    def parent(open_tag, tag, fill):
        # an element without children prints as one empty-element tag
        start = len(x)
        fill()
        if len(x) == start:
            x.append("            <%s />\n" % open_tag)
        else:
            x.insert(start, "            <%s>\n" % open_tag)
            x.append("            </%s>\n" % tag)

    def vertex_children():
        element(ind, "Coord", "coord", coords, True)
        if normal_type == "vertex":
            element(ind, "Normal", "normal", normals, True)

    def polygon_children():
        element(ind, "Connection", "connect", conn, False)
        value(ind, "Color", color)
        value(ind, "Opacity", opacity)
        if normal_type != "vertex":
            element(ind, "Normal", "normal", normals, True)

    parent('Vertex nvertices="%d"' % nv, "Vertex", vertex_children)
    parent('Polygon npolygons="%d"' % npoly, "Polygon", polygon_children)
    x.append("        </PolygonObject>\n    </Object>\n</KVSML>\n")
    files[base + ".kvsml"] = "".join(x).encode()
    return files
