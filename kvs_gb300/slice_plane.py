"""kvs::SlicePlane on the GPU: structured volumes (kvsmc_slice_plane) and
unstructured ones (kvsmc_slice_cells_host).

Mirrors the reference mapper (Source/Core/Visualization/Mapper/SlicePlane.h,
SlicePlane.cpp): the two constructor forms (coefficients, or a point and a
normal), the exec/mapping checks and messages, MapperBase::setRange for the
colour map and setMinMaxCoords for the bounding box, and the same
PolygonObject: duplicated triangles in cell order, one RGB colour per vertex
(VertexColor), one normal per triangle (PolygonNormal), opacity 255.  All
per-cell work runs in libkvsmc's CUDA kernels.  As in the reference, the
mapper's success flag is never set true (MapperBase starts false); a GPU
failure is reported and exec returns None.  An UnstructuredVolumeObject of
tetrahedra, hexahedra, pyramids or prisms is sliced per cell by its cell
type's marching table (SlicePlane.cpp:291-800, node coordinates as they are);
other cell types give nothing, as in the reference.
"""
import numpy as np

from . import _abi
from .marching_cells import MAPPERS, UnstructuredVolumeObject, set_bounds_on_device
from .marching_cubes import (PolygonObject, StructuredVolumeObject, TransferFunction, _equal, default_context,
                             message_error, set_mapper_range)

f32 = np.float32


class SlicePlane(PolygonObject):
    """kvs::SlicePlane (structured volumes on the GPU)."""

    def __init__(self, volume=None, coefficients=None, point=None, normal=None, transfer_function=None,
                 context=None):
        super().__init__()
        self._tfunc = (transfer_function or TransferFunction(256)).copy()
        self._coef = np.zeros(4, f32)
        self._ctx = context
        self._success = False        # MapperBase() (MapperBase.cpp:23)
        self.ntriangles = 0
        if coefficients is not None or point is not None:
            self.setPlane(coefficients=coefficients, point=point, normal=normal)
        if volume is not None:
            self.exec(volume)

    def setPlane(self, coefficients=None, point=None, normal=None):
        """SlicePlane::setPlane (SlicePlane.h:50-51): coefficients, or
        (normal, -point.dot(normal)) in float."""
        if coefficients is not None:
            self._coef = np.asarray(coefficients, f32).copy()
            return
        p, n = np.asarray(point, f32), np.asarray(normal, f32)
        dot = f32(f32(f32(p[0] * n[0]) + f32(p[1] * n[1])) + f32(p[2] * n[2]))
        self._coef = np.array([n[0], n[1], n[2], -dot], f32)

    def coefficients(self):
        return self._coef

    def setTransferFunction(self, tfunc):
        self._tfunc = tfunc.copy()

    def transferFunction(self):
        return self._tfunc

    def isSuccess(self):
        return self._success

    def isFailure(self):
        return not self._success

    def exec(self, obj):
        """SlicePlane::exec (SlicePlane.cpp:60-80)."""
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, (StructuredVolumeObject, UnstructuredVolumeObject)):
            self._success = False
            message_error("Input object is not volume dat.")
            return None
        try:
            self._mapping(obj)
        except _abi.KvsmcError as e:
            self._success = False
            message_error(f"libkvsmc: {e}")
            return None
        return self

    def _set_range(self, code, volume):
        """MapperBase::setRange (MapperBase.cpp:54-83), the volume's min/max
        cache filled first."""
        set_mapper_range(self._tfunc, code, volume.minValue(), volume.maxValue())

    def _mapping_cells(self, volume):
        """SlicePlane::mapping, unstructured branch (SlicePlane.cpp:128-147, 291-320)."""
        values = volume.values()
        try:
            code = _abi.dtype_code(values.dtype)
        except TypeError:
            code = None
        mapper = MAPPERS.get(volume.cellType())
        ctx = self._ctx or default_context()
        n = volume.numberOfNodes()
        conn = volume.connections()[:volume.numberOfCells() * volume.numberOfCellNodes()]
        if mapper is not None and code is not None and not volume.hasMinMaxValues():
            # UnstructuredVolumeObject::updateMinMaxValues by the device scan
            _, _, sizes = _abi.marching_cells_host(ctx, mapper.ABI_CELL, values[:n], volume.coords()[:3 * n], conn,
                                                   float("nan"))
            volume.setMinMaxValues(sizes["min_value"], sizes["max_value"])
        self._set_range(code, volume)
        if not volume.hasMinMaxObjectCoords():
            if mapper is not None:
                set_bounds_on_device(ctx, volume, mapper.ABI_CELL, conn)
            else:
                volume.updateMinMaxCoords()
        self.setMinMaxObjectCoords(volume.minObjectCoord(), volume.maxObjectCoord())
        self.setMinMaxExternalCoords(volume.minExternalCoord(), volume.maxExternalCoord())
        if code is None:
            self._success = False
            message_error(f"Unsupported data type '{values.dtype}'.")
            return
        if mapper is None:
            return                      # extract_plane: default: break
        p = _abi.SliceParams()
        for k in range(4):
            p.coefficients[k] = float(self._coef[k])
        table = np.ascontiguousarray(self._tfunc.table, np.uint8)
        p.tf_min, p.tf_max = float(self._tfunc.min_value), float(self._tfunc.max_value)
        p.tf_resolution = table.shape[0]
        p.tf_table = table.ctypes.data
        coords, normals, colors, ntri = slice_cells_host(ctx, mapper.ABI_CELL, values[:n], volume.coords()[:3 * n],
                                                         conn, p)
        self._coords = coords
        self._colors = colors
        self._normals = normals
        self._opacities = np.array([255], np.uint8)
        self._polygon_type = PolygonObject.Triangle
        self._color_type = PolygonObject.VertexColor
        self._normal_type = PolygonObject.PolygonNormal
        self.ntriangles = ntri

    def _mapping(self, volume):
        """SlicePlane::mapping (SlicePlane.cpp:88-145)."""
        if volume.veclen() != 1:
            self._success = False
            message_error("Input volume is not a sclar field data.")
            return
        if isinstance(volume, UnstructuredVolumeObject):
            return self._mapping_cells(volume)
        values = volume.values()
        try:
            code = _abi.dtype_code(values.dtype)
        except TypeError:
            self._success = False
            message_error(f"Unsupported data type '{values.dtype}'.")
            return
        ctx = self._ctx or default_context()
        dv = _abi.DeviceVolume.upload(ctx, volume.volume_array())
        try:
            # MapperBase::setRange (MapperBase.cpp:54-83): the cache first
            if not volume.hasMinMaxValues():
                volume.setMinMaxValues(*dv.minmax())
            self._set_range(code, volume)
            # MapperBase::setMinMaxCoords (MapperBase.cpp:92-122)
            if not volume.hasMinMaxObjectCoords():
                volume.updateMinMaxCoords()
            self.setMinMaxObjectCoords(volume.minObjectCoord(), volume.maxObjectCoord())
            self.setMinMaxExternalCoords(volume.minExternalCoord(), volume.maxExternalCoord())
            nx, ny, nz = volume.resolution()
            mn, mx = volume.minObjectCoord(), volume.maxObjectCoord()
            p = _abi.SliceParams()
            for k in range(4):
                p.coefficients[k] = float(self._coef[k])
            with np.errstate(divide="ignore", invalid="ignore"):
                for k, n in enumerate((nx, ny, nz)):
                    p.min_coord[k] = float(mn[k])
                    p.scale[k] = float(f32(f32(mx[k] - mn[k]) / f32(n - 1)))
            table = np.ascontiguousarray(self._tfunc.table, np.uint8)
            p.tf_min, p.tf_max = float(self._tfunc.min_value), float(self._tfunc.max_value)
            p.tf_resolution = table.shape[0]
            p.tf_table = table.ctypes.data
            coords, normals, colors, n = slice_plane_host(ctx, dv, p)
        finally:
            dv.free()
        # SlicePlane.cpp:196-202
        self._coords = coords
        self._colors = colors
        self._normals = normals
        self._opacities = np.array([255], np.uint8)
        self._polygon_type = PolygonObject.Triangle
        self._color_type = PolygonObject.VertexColor
        self._normal_type = PolygonObject.PolygonNormal
        self.ntriangles = n


def slice_plane_host(ctx, dv, params):
    """kvsmc_slice_plane on a DeviceVolume: (coords, normals, colours, triangles)."""
    import ctypes as C
    bufs = {}

    def alloc(user, which, count):
        a = np.empty(count, dtype=np.uint8 if which == 3 else np.float32)
        bufs[which] = a
        return a.ctypes.data

    cb = _abi.HOST_ALLOC(alloc)
    n = C.c_uint64(0)
    ctx.check(ctx.lib.kvsmc_slice_plane(ctx.handle, dv.handle, C.byref(params), cb, None, C.byref(n)),
              "kvsmc_slice_plane")
    return (bufs.get(0, np.zeros(0, f32)), bufs.get(1, np.zeros(0, f32)), bufs.get(3, np.zeros(0, np.uint8)),
            n.value)


def slice_cells_host(ctx, cell_type, values, coords, connections, params):
    """kvsmc_slice_cells_host: (coords, normals, colours, triangles) of one unstructured volume."""
    import ctypes as C
    v = np.ascontiguousarray(values).reshape(-1)
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(connections, np.uint32).reshape(-1)
    npc = _abi.CELL_NODES[int(cell_type)]
    bufs = {}

    def alloc(user, which, count):
        a = np.empty(count, dtype=np.uint8 if which == 3 else np.float32)
        bufs[which] = a
        return a.ctypes.data

    cb = _abi.HOST_ALLOC(alloc)
    n = C.c_uint64(0)
    ctx.check(ctx.lib.kvsmc_slice_cells_host(ctx.handle, int(cell_type), v.ctypes.data, _abi.dtype_code(v.dtype),
                                             v.size, c.ctypes.data, k.ctypes.data if k.size else None,
                                             k.size // npc, C.byref(params), cb, None, C.byref(n)),
              "kvsmc_slice_cells_host")
    return (bufs.get(0, np.zeros(0, f32)), bufs.get(1, np.zeros(0, f32)), bufs.get(3, np.zeros(0, np.uint8)),
            n.value)
