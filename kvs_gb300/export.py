"""Binary STL export of triangle meshes, serialised on the GPU.

Mirrors kvs::PolygonExporter<kvs::Stl> (Source/Core/Visualization/Exporter/
PolygonExporter.h:53-61, PolygonExporter.cpp:78-176) with kvs::Stl's Binary
file type (Source/Core/FileFormat/STL/Stl.cpp:490-540): the same checks and
messages, the same bytes.  The records are formed by libkvsmc's CUDA kernel
(kvsmc_stl_records); a mesh already on the device (kvsmc_extract_device
output) is written without any host PolygonObject (write_stl_device).

The reference's kvs::Stl defaults to ASCII; ASCII output is not provided here
(write() reports it and returns False): set the Binary file type.
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
        """Stl::write (Stl.cpp:170-199) with the Binary file type."""
        if self._mesh is None:
            message_error("No polygon object to write.")
            return False
        if self._file_type != BINARY:
            message_error("ASCII STL is not provided; setFileType('binary').")
            return False
        m = self._mesh
        ctx = self._ctx or default_context()
        c = np.ascontiguousarray(m.coords(), np.float32)
        n = np.ascontiguousarray(m.normals(), np.float32)
        k = np.ascontiguousarray(m.connections(), np.uint32)
        st = ctx.lib.kvsmc_write_stl_host(ctx.handle, str(filename).encode(), _mode(m), c.ctypes.data, c.size,
                                          n.ctypes.data, n.size, k.ctypes.data if k.size else None, k.size)
        if st:
            message_error(f"libkvsmc: {_abi.status_string(st)}: {ctx.lib.kvsmc_last_error(ctx.handle).decode()}")
            self._success = False
            return False
        return True
