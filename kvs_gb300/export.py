"""Binary STL and PLY export of triangle meshes, serialised on the GPU.

Mirrors kvs::PolygonExporter<kvs::Stl> (Source/Core/Visualization/Exporter/
PolygonExporter.h:53-61, PolygonExporter.cpp:78-176) with kvs::Stl's Binary
file type (Source/Core/FileFormat/STL/Stl.cpp:490-540): the same checks and
messages, the same bytes.  The records are formed by libkvsmc's CUDA kernel
(kvsmc_stl_records); a mesh already on the device (kvsmc_extract_device
output) is written without any host PolygonObject (write_stl_device).

kvs::Stl's default ASCII file type (Stl.cpp:86, write_ascii :447-480) is
formatted on the GPU too (kvsmc_write_stl_ascii: exact "%f" text, byte for
byte the reference's file).

PolygonExporterKVSML mirrors kvs::PolygonExporter<kvs::KVSMLPolygonObject>
(PolygonExporter.cpp:22-68) + KVSMLPolygonObject::write (KVSMLPolygonObject.cpp:
349-492) with its three writing data types (kvsmc_write_kvsml_polygon).

PolygonExporterPly mirrors kvs::PolygonExporter<kvs::Ply> (PolygonExporter.cpp:
178-361) with kvs::Ply's Binary type (Ply.cpp:389-488) for meshes without
connections (the reference's writer cannot store faces); the vertex records
are formed by kvsmc_write_ply's kernel.  The reference's writer aborts while
freeing its element tables after the file is closed (PlyFile.cpp:1345-1366:
the never-described face element's property array); the file it leaves is
complete, and that file is what this writer reproduces.
"""
import numpy as np

from . import _abi
from .marching_cubes import PolygonObject, default_context, message_error

ASCII, BINARY = 0, 1


def _mode(polygon):
    if polygon.numberOfConnections() == 0:
        return _abi.MODE_DUP_POLYGON_NORMAL
    if polygon.normalType() == PolygonObject.VertexNormal:
        return _abi.MODE_SHARED_VERTEX_NORMAL
    return _abi.MODE_SHARED_POLYGON_NORMAL


def stl_records_device(ctx, mode, d_coords, d_normals, d_connections, nvertices, ntriangles, d_out):
    """kvsmc_stl_records: 50-byte records of a device mesh into d_out (device
    pointers as integers)."""
    ctx.check(ctx.lib.kvsmc_stl_records(ctx.handle, int(mode), d_coords, d_normals, d_connections or None,
                                        int(nvertices), int(ntriangles), d_out), "stl_records")


def write_stl_device(ctx, path, mode, d_coords, d_normals, d_connections, nvertices, ntriangles):
    """kvsmc_write_stl: the binary STL file of a device mesh."""
    ctx.check(ctx.lib.kvsmc_write_stl(ctx.handle, str(path).encode(), int(mode), d_coords, d_normals,
                                      d_connections or None, int(nvertices), int(ntriangles)), "write_stl")


class PolygonExporterStl:
    """kvs::PolygonExporter<kvs::Stl>: exec(polygon) keeps the mesh, write()
    serialises it on the GPU."""

    def __init__(self, polygon=None, context=None):
        self._success = True
        self._file_type = ASCII          # kvs::Stl() (Stl.cpp:85-89)
        self._mesh = None
        self._ctx = context
        if polygon is not None:
            self.exec(polygon)

    def isSuccess(self):
        return self._success

    def isFailure(self):
        return not self._success

    def setFileType(self, file_type):
        self._file_type = BINARY if file_type in (BINARY, "binary", "Binary") else ASCII

    def fileType(self):
        return self._file_type

    def exec(self, obj):
        """PolygonExporter<kvs::Stl>::exec (PolygonExporter.cpp:78-99)."""
        self._success = True
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, PolygonObject):
            self._success = False
            message_error("Input object is not polygon object.")
            return None
        if obj.polygonType() != PolygonObject.Triangle:
            self._success = False
            message_error("Input object is not triangle polygon.")
            return None
        self._mesh = obj
        return self

    def write(self, filename):
        """Stl::write (Stl.cpp:170-199): the ASCII (default) or Binary file type."""
        if self._mesh is None:
            message_error("No polygon object to write.")
            return False
        m = self._mesh
        ctx = self._ctx or default_context()
        c = np.ascontiguousarray(m.coords(), np.float32)
        n = np.ascontiguousarray(m.normals(), np.float32)
        k = np.ascontiguousarray(m.connections(), np.uint32)
        fn = ctx.lib.kvsmc_write_stl_host if self._file_type == BINARY else ctx.lib.kvsmc_write_stl_ascii_host
        st = fn(ctx.handle, str(filename).encode(), _mode(m), c.ctypes.data, c.size,
                n.ctypes.data, n.size, k.ctypes.data if k.size else None, k.size)
        if st:
            message_error(f"libkvsmc: {_abi.status_string(st)}: {ctx.lib.kvsmc_last_error(ctx.handle).decode()}")
            self._success = False
            return False
        return True


def write_stl_ascii_device(ctx, path, mode, d_coords, d_normals, d_connections, nvertices, ntriangles):
    """kvsmc_write_stl_ascii: the ASCII STL file of a device mesh, text formatted on the GPU."""
    ctx.check(ctx.lib.kvsmc_write_stl_ascii(ctx.handle, str(path).encode(), int(mode), d_coords, d_normals,
                                            d_connections or None, int(nvertices), int(ntriangles)),
              "write_stl_ascii")


# ------------------------------------------------------------------ KVSML

KVSML_ASCII, KVSML_EXTERNAL_ASCII, KVSML_EXTERNAL_BINARY = 0, 1, 2


def write_kvsml_device(ctx, path, writing_type, mode, d_coords, ncoords, d_normals, nnormals, d_connections,
                       nconnections, color=None, opacity=None):
    """kvsmc_write_kvsml_polygon on device arrays (pointers as integers, sizes in elements)."""
    col = np.ascontiguousarray(color, np.uint8) if color is not None and len(color) == 3 else None
    opa = np.ascontiguousarray(opacity, np.uint8).reshape(-1)[:1] if opacity is not None and len(opacity) else None
    ctx.check(ctx.lib.kvsmc_write_kvsml_polygon(ctx.handle, str(path).encode(), int(writing_type), int(mode),
                                                d_coords or None, int(ncoords), d_normals or None, int(nnormals),
                                                d_connections or None, int(nconnections),
                                                col.ctypes.data if col is not None else None,
                                                opa.ctypes.data if opa is not None else None), "write_kvsml")


class PolygonExporterKVSML:
    """kvs::PolygonExporter<kvs::KVSMLPolygonObject>: exec(polygon) keeps the
    mesh, write() writes the .kvsml file (and its external data files)."""

    def __init__(self, polygon=None, context=None):
        self._success = True
        self._writing = KVSML_ASCII      # KVSMLPolygonObject() (KVSMLPolygonObject.cpp:33-39)
        self._mesh = None
        self._ctx = context
        if polygon is not None:
            self.exec(polygon)

    def isSuccess(self):
        return self._success

    def setWritingDataTypeToAscii(self):
        self._writing = KVSML_ASCII

    def setWritingDataTypeToExternalAscii(self):
        self._writing = KVSML_EXTERNAL_ASCII

    def setWritingDataTypeToExternalBinary(self):
        self._writing = KVSML_EXTERNAL_BINARY

    def exec(self, obj):
        """PolygonExporter<KVSMLPolygonObject>::exec (PolygonExporter.cpp:22-68)."""
        self._success = True
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, PolygonObject):
            self._success = False
            message_error("Input object is not polygon object.")
            return None
        self._mesh = obj
        return self

    def write(self, filename):
        """KVSMLPolygonObject::write (KVSMLPolygonObject.cpp:349-492)."""
        if self._mesh is None:
            message_error("No polygon object to write.")
            return False
        m = self._mesh
        if m.polygonType() != PolygonObject.Triangle or m.colorType() != PolygonObject.PolygonColor:
            message_error("KVSML: triangle meshes with one polygon colour are provided")
            self._success = False
            return False
        import torch
        ctx = self._ctx or default_context()
        c = torch.from_numpy(np.ascontiguousarray(m.coords(), np.float32)).cuda()
        n = torch.from_numpy(np.ascontiguousarray(m.normals(), np.float32)).cuda()
        k = torch.from_numpy(np.ascontiguousarray(m.connections(), np.uint32).view(np.int32)).cuda()
        mode = (_abi.MODE_SHARED_VERTEX_NORMAL if m.normalType() == PolygonObject.VertexNormal
                else _abi.MODE_DUP_POLYGON_NORMAL)
        col = m.colors()
        opa = m.opacities() if hasattr(m, "opacities") else np.array([m.opacity()], np.uint8)
        try:
            write_kvsml_device(ctx, filename, self._writing, mode, c.data_ptr() if c.numel() else None, c.numel(),
                               n.data_ptr() if n.numel() else None, n.numel(), k.data_ptr() if k.numel() else None,
                               k.numel(), col if len(col) == 3 else None, opa)
        except _abi.KvsmcError as e:
            message_error(str(e))
            self._success = False
            return False
        return True


# ------------------------------------------------------------------ PLY

def ply_modes(polygon):
    """(colour mode, normal mode) of kvsmc_write_ply for a connection-less
    triangle mesh, as PolygonExporter<kvs::Ply>::exec (PolygonExporter.cpp:
    208-357) forms the vertex colours and normals; raises ValueError where the
    reference gives no defined output."""
    if polygon.numberOfConnections() > 0:
        raise ValueError("meshes with connections: the reference's PLY writer stores face indices through a "
                         "null pointer (Ply.cpp:470-480)")
    ncol = polygon.colors().size
    if ncol == 0:
        cm = 0
    elif ncol == 3:
        cm = 1                                     # the single colour on every vertex (:208-219)
    elif polygon.colorType() == PolygonObject.VertexColor:
        cm = 2                                     # the vertex colours as they are (:302-305)
    else:
        raise ValueError("per-polygon colours: the reference sets only the red channel of the averaged vertex "
                         "colours and leaves green and blue uninitialised (PolygonExporter.cpp:254-258)")
    if polygon.normals().size == 0:
        nm = 0
    elif polygon.normalType() == PolygonObject.PolygonNormal:
        nm = 1                                     # averaged over connections, of which there are none: zeros
    else:
        nm = 2                                     # the vertex normals as they are (:350-353)
    return cm, nm


def write_ply_device(ctx, path, d_coords, nvertices, d_colors, color_mode, d_normals, normal_mode):
    """kvsmc_write_ply: the binary PLY file of a device mesh (device pointers as integers)."""
    ctx.check(ctx.lib.kvsmc_write_ply(ctx.handle, str(path).encode(), d_coords, int(nvertices), d_colors or None,
                                      int(color_mode), d_normals or None, int(normal_mode)), "write_ply")


class PolygonExporterPly:
    """kvs::PolygonExporter<kvs::Ply>: exec(polygon) keeps the mesh, write()
    serialises it (binary, little endian) on the GPU."""

    def __init__(self, polygon=None, context=None):
        self._success = True
        self._file_type = ASCII          # kvs::Ply() (Ply.cpp:96-103)
        self._mesh = None
        self._ctx = context
        if polygon is not None:
            self.exec(polygon)

    def isSuccess(self):
        return self._success

    def isFailure(self):
        return not self._success

    def setFileType(self, file_type):
        self._file_type = BINARY if file_type in (BINARY, "binary", "Binary") else ASCII

    def fileType(self):
        return self._file_type

    def exec(self, obj):
        """PolygonExporter<kvs::Ply>::exec (PolygonExporter.cpp:178-200)."""
        self._success = True
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, PolygonObject):
            self._success = False
            message_error("Input object is not polygon object.")
            return None
        if obj.polygonType() != PolygonObject.Triangle:
            self._success = False
            message_error("Input object is not triangle polygon.")
            return None
        self._mesh = obj
        return self

    def write(self, filename):
        """Ply::write (Ply.cpp:389-488) with the Binary file type."""
        if self._mesh is None:
            message_error("No polygon object to write.")
            return False
        if self._file_type != BINARY:
            message_error("ASCII PLY is not provided; setFileType('binary').")
            return False
        m = self._mesh
        try:
            cm, nm = ply_modes(m)
        except ValueError as e:
            message_error(f"PLY: {e}")
            self._success = False
            return False
        ctx = self._ctx or default_context()
        c = np.ascontiguousarray(m.coords(), np.float32)
        k = np.ascontiguousarray(m.colors(), np.uint8)
        n = np.ascontiguousarray(m.normals(), np.float32)
        nv = c.size // 3
        if (cm == 2 and k.size < 3 * nv) or (nm == 2 and n.size < 3 * nv):
            message_error("PLY: fewer vertex colours / normals than vertices")
            self._success = False
            return False
        st = ctx.lib.kvsmc_write_ply_host(ctx.handle, str(filename).encode(), c.ctypes.data, nv,
                                          k.ctypes.data if cm else None, cm, n.ctypes.data if nm == 2 else None, nm)
        if st:
            message_error(f"libkvsmc: {_abi.status_string(st)}: {ctx.lib.kvsmc_last_error(ctx.handle).decode()}")
            self._success = False
            return False
        return True
