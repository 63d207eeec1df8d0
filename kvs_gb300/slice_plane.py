"""kvs::SlicePlane for structured volumes, on the GPU (kvsmc_slice_plane).

Mirrors the reference mapper (Source/Core/Visualization/Mapper/SlicePlane.h,
SlicePlane.cpp): the two constructor forms (coefficients, or a point and a
normal), the exec/mapping checks and messages, MapperBase::setRange for the
colour map and setMinMaxCoords for the bounding box, and the same
PolygonObject: duplicated triangles in cell order, one RGB colour per vertex
(VertexColor), one normal per triangle (PolygonNormal), opacity 255.  All
per-cell work runs in libkvsmc's CUDA kernels.  As in the reference, the
mapper's success flag is never set true (MapperBase starts false); a GPU
failure is reported and exec returns None.  Unstructured volumes are not
handled by this package.
"""
import numpy as np

from . import _abi
from .marching_cubes import (PolygonObject, StructuredVolumeObject, TransferFunction, _equal, default_context,
                             message_error)

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
        if not isinstance(obj, StructuredVolumeObject):
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

    def _mapping(self, volume):
        """SlicePlane::mapping (SlicePlane.cpp:88-145), structured branch."""
        if volume.veclen() != 1:
            self._success = False
            message_error("Input volume is not a sclar field data.")
            return
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
            # MapperBase::setRange (MapperBase.cpp:54-83)
            if not self._tfunc.hasRange():
                if code == 0:
                    self._tfunc.setRange(-128, 127)
                elif code == 4:
                    self._tfunc.setRange(0, 255)
                else:
                    if not volume.hasMinMaxValues():
                        volume.setMinMaxValues(*dv.minmax())
                    lo, hi = f32(volume.minValue()), f32(volume.maxValue())
                    self._tfunc.setRange(lo, hi + f32(1.0) if _equal(float(lo), float(hi)) else hi)
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
