"""Host-side mirror of the reference mapper interface, over libkvsmc.

The classes keep the reference's names, argument meaning and error behaviour
(Source/Core/Visualization/...):

  StructuredVolumeObject  Object/StructuredVolumeObject.h:23-99 (input)
  PolygonObject           Object/PolygonObject.h:27-96        (output)
  TransferFunction        Mapper/TransferFunction.cpp:39-45   (colour only)
  MarchingCubes           Mapper/MarchingCubes.h:23-62        (the mapper)

All per-cell work (min/max scan, classification, interpolation, normals,
compaction in the reference's order) runs in libkvsmc's CUDA kernels; this
module only decides what the reference decides on the host (ranges, bounding
box, early exits, colour) and copies arrays.  There is no CPU fallback: if
libkvsmc.so is missing or no GPU is present, exec() fails loudly.
"""
import sys

import numpy as np

from . import _abi
from .default_colormap import BREWER_RDBU_256

_TINY = 1.0e-6


def _equal(a, b):
    """kvs::Math::Equal (Utility/Math.h:135-138)."""
    d = a - b
    return (-d if d < 0 else d) < _TINY


def message_error(text):
    """kvsMessageError (Utility/Message.h:25): report and carry on."""
    print(f"KVS ERROR: {text}", file=sys.stderr)


class ObjectBase:
    """Bounding-box part of kvs::ObjectBase (Object/ObjectBase.h:44-77)."""

    def __init__(self):
        self._min_obj = np.zeros(3, np.float32)
        self._max_obj = np.zeros(3, np.float32)
        self._min_ext = np.zeros(3, np.float32)
        self._max_ext = np.zeros(3, np.float32)
        self._has_obj = False
        self._has_ext = False

    def setMinMaxObjectCoords(self, mn, mx):
        self._min_obj = np.asarray(mn, np.float32).copy()
        self._max_obj = np.asarray(mx, np.float32).copy()
        self._has_obj = True

    def setMinMaxExternalCoords(self, mn, mx):
        self._min_ext = np.asarray(mn, np.float32).copy()
        self._max_ext = np.asarray(mx, np.float32).copy()
        self._has_ext = True

    def hasMinMaxObjectCoords(self):
        return self._has_obj

    def hasMinMaxExternalCoords(self):
        return self._has_ext

    def minObjectCoord(self):
        return self._min_obj

    def maxObjectCoord(self):
        return self._max_obj

    def minExternalCoord(self):
        return self._min_ext

    def maxExternalCoord(self):
        return self._max_ext


class StructuredVolumeObject(ObjectBase):
    """kvs::StructuredVolumeObject: values x fastest; `values` may be given
    shaped (nz, ny, nx) or flat with setResolution((nx, ny, nz))."""

    UnknownGridType, Uniform, Rectilinear, Curvilinear = 0, 1, 2, 3

    def __init__(self, values=None, resolution=None, veclen=1, grid_type=1, coords=None):
        super().__init__()
        self._values = None
        self._resolution = (0, 0, 0)
        self._veclen = veclen
        self._grid_type = grid_type
        self._coords = None if coords is None else np.asarray(coords, np.float32)
        self._has_minmax = False
        self._min_value = 0.0
        self._max_value = 0.0
        if values is not None:
            self.setValues(values)
        if resolution is not None:
            self.setResolution(resolution)

    # setters (StructuredVolumeObject.h:44-52, VolumeObjectBase.h:60-68)
    def setValues(self, values):
        v = np.asarray(values)
        if v.ndim == 3:
            self._resolution = (v.shape[2], v.shape[1], v.shape[0])
        self._values = np.ascontiguousarray(v).reshape(-1)

    def setResolution(self, res):
        self._resolution = tuple(int(r) for r in res)

    def setVeclen(self, veclen):
        self._veclen = int(veclen)

    def setGridType(self, t):
        self._grid_type = t

    def setGridTypeToUniform(self):
        self._grid_type = self.Uniform

    def setGridTypeToRectilinear(self):
        self._grid_type = self.Rectilinear

    def setCoords(self, coords):
        self._coords = np.asarray(coords, np.float32)

    def setMinMaxValues(self, mn, mx):
        self._min_value, self._max_value, self._has_minmax = float(mn), float(mx), True

    # getters
    def values(self):
        return self._values

    def resolution(self):
        return self._resolution

    def veclen(self):
        return self._veclen

    def gridType(self):
        return self._grid_type

    def hasMinMaxValues(self):
        return self._has_minmax

    def minValue(self):
        return self._min_value

    def maxValue(self):
        return self._max_value

    def numberOfNodes(self):
        nx, ny, nz = self._resolution
        return nx * ny * nz

    def volume_array(self):
        nx, ny, nz = self._resolution
        return self._values.reshape(nz, ny, nx)

    def updateMinMaxCoords(self):
        """StructuredVolumeObject.cpp:348-423 (uniform and rectilinear grids)."""
        nx, ny, nz = self._resolution
        mn = np.zeros(3, np.float32)
        mx = np.zeros(3, np.float32)
        if self._grid_type == self.Uniform:
            mx = np.array([np.float32(nx) - np.float32(1), np.float32(ny) - np.float32(1),
                           np.float32(nz) - np.float32(1)], np.float32)
        elif self._grid_type == self.Rectilinear:
            c = self._coords
            mn = np.array([c[0], c[nx], c[nx + ny]], np.float32)
            mx = np.array([c[nx - 1], c[nx + ny - 1], c[nx + ny + nz - 1]], np.float32)
        elif self._grid_type == self.Curvilinear:
            c = self._coords.reshape(-1, 3)
            mn, mx = c.min(axis=0).astype(np.float32), c.max(axis=0).astype(np.float32)
        self.setMinMaxObjectCoords(mn, mx)
        if not self.hasMinMaxExternalCoords():
            self.setMinMaxExternalCoords(self.minObjectCoord(), self.maxObjectCoord())


class PolygonObject(ObjectBase):
    """Output arrays of kvs::PolygonObject (Object/PolygonObject.h:27-96)."""

    Triangle, Quadrangle = 3, 4
    VertexColor, PolygonColor = 0, 1
    VertexNormal, PolygonNormal = 0, 1

    def __init__(self):
        super().__init__()
        self._coords = np.zeros(0, np.float32)
        self._normals = np.zeros(0, np.float32)
        self._connections = np.zeros(0, np.uint32)
        self._colors = np.zeros(0, np.uint8)           # no colour until a mapper sets one
        self._opacities = np.array([255], np.uint8)   # PolygonObject.cpp:154-157
        self._polygon_type = 5                         # UnknownPolygonType
        self._normal_type = 2                          # UnknownNormalType
        self._color_type = 2                           # UnknownColorType

    def coords(self):
        return self._coords

    def normals(self):
        return self._normals

    def connections(self):
        return self._connections

    def colors(self):
        return self._colors

    def opacities(self):
        return self._opacities

    def polygonType(self):
        return self._polygon_type

    def normalType(self):
        return self._normal_type

    def colorType(self):
        return self._color_type

    def setNormalType(self, t):
        self._normal_type = t

    def numberOfVertices(self):
        return self._coords.size // 3

    def numberOfConnections(self):
        return self._connections.size // 3


class TransferFunction:
    """The colour part of kvs::TransferFunction: a resolution x RGB table and
    an optional range.  Default: the reference's BrewerRdBu table at 256."""

    def __init__(self, resolution=256, table=None):
        self.resolution = int(resolution)
        if table is None:
            if self.resolution != 256:
                raise ValueError("only the default 256-entry colour map is built in; pass `table`")
            table = np.frombuffer(BREWER_RDBU_256, np.uint8).reshape(256, 3)
        self.table = np.asarray(table, np.uint8).reshape(-1, 3)
        self.min_value = np.float32(0.0)
        self.max_value = np.float32(0.0)

    def setRange(self, mn, mx):
        self.min_value, self.max_value = np.float32(mn), np.float32(mx)

    def hasRange(self):
        """ColorMap::hasRange (ColorMap.cpp:850-853)."""
        return not _equal(float(self.min_value), float(self.max_value))

    def copy(self):
        t = TransferFunction(self.resolution, self.table.copy())
        t.min_value, t.max_value = self.min_value, self.max_value
        return t

    def color_at(self, value):
        """ColorMap::at (ColorMap.cpp:1043-1054) with RGBColor::Mix in float."""
        f32 = np.float32
        lo, hi = self.min_value, self.max_value
        value = f32(value)
        v0 = lo if value <= lo else (value if value <= hi else hi)
        r = f32(self.resolution - 1)
        with np.errstate(invalid="ignore", divide="ignore"):
            v = f32(f32(f32(v0 - lo) / f32(hi - lo)) * r)
        if not np.isfinite(v):
            # the reference converts a NaN/inf table position to size_t, which is
            # undefined behaviour in C++ (a NaN value range); use entry 0 here
            v = f32(0.0)
        s0 = int(v)
        s1 = min(s0 + 1, self.resolution - 1)
        t = f32(v - f32(s0))
        out = np.zeros(3, np.uint8)
        for k in range(3):
            a = f32(f32(self.table[s0, k]) / f32(255.0))
            b = f32(f32(self.table[s1, k]) / f32(255.0))
            m = f32(f32(a * f32(f32(1) - t)) + f32(b * t))
            m = f32(0.0) if m <= 0 else (m if m <= 1 else f32(1.0))
            x = float(f32(m * f32(255.0)))
            out[k] = int(x + 0.5) if x >= 0 else -int(0.5 - x)
        return out


def set_mapper_range(tfunc, code, vmin, vmax):
    """MapperBase::setRange (MapperBase.cpp:54-83) for a transfer function
    without a range: int8 and uint8 volumes take their type's range (dtype
    codes 0 and 4), the others the volume's min/max as floats, widened by 1
    when kvs::Math::Equal calls them equal."""
    if tfunc.hasRange():
        return
    if code == 0:
        tfunc.setRange(-128, 127)
    elif code == 4:
        tfunc.setRange(0, 255)
    else:
        f32 = np.float32
        lo, hi = f32(vmin), f32(vmax)
        tfunc.setRange(lo, hi + f32(1.0) if _equal(float(lo), float(hi)) else hi)


_context = None


def default_context():
    global _context
    if _context is None:
        _context = _abi.Context()
    return _context


class MarchingCubes(PolygonObject):
    """kvs::cuda::MarchingCubes: drop-in for kvs::MarchingCubes.

    MarchingCubes(volume, isolevel, normal_type, duplication, transfer_function)
    runs exec(volume) immediately, like the reference constructor
    (MarchingCubes.cpp:25-37); MarchingCubes() + setIsolevel/... + exec() is
    the pipeline-module form."""

    def __init__(self, volume=None, isolevel=0.0, normal_type=PolygonObject.PolygonNormal,
                 duplication=True, transfer_function=None, context=None):
        super().__init__()
        self._tfunc = (transfer_function or TransferFunction(256)).copy()
        self._isolevel = float(isolevel)
        self._duplication = bool(duplication)
        self._volume = None
        self._success = False
        self._ctx = context
        self.sizes = None
        self.setNormalType(normal_type)
        if volume is not None:
            self.exec(volume)

    # MapperBase (Mapper/MapperBase.h:26-63)
    def setIsolevel(self, isolevel):
        self._isolevel = float(isolevel)

    def setTransferFunction(self, tfunc):
        self._tfunc = tfunc.copy()

    def transferFunction(self):
        return self._tfunc

    def isSuccess(self):
        return self._success

    def isFailure(self):
        return not self._success

    def exec(self, obj):
        """MarchingCubes::exec (MarchingCubes.cpp:46-79)."""
        self._success = False
        if obj is None:
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, StructuredVolumeObject):
            message_error("Input object is not structured volume object.")
            return None
        if obj.veclen() != 1:
            message_error("Input volume is not sclar field data.")
            return None
        if self.normalType() == PolygonObject.VertexNormal:
            self._duplication = False
        try:
            self._mapping(obj)
        except _abi.KvsmcError as e:
            # no CPU fallback: the GPU call failed, so the mapper failed
            message_error(f"libkvsmc: {e}")
            return None
        self._success = True
        return self

    def _mapping(self, volume):
        """MarchingCubes::mapping (MarchingCubes.cpp:87-132)."""
        self._volume = volume
        values = volume.values()
        try:
            code = _abi.dtype_code(values.dtype)
        except TypeError:
            message_error(f"Unsupported data type '{values.dtype}'.")
            return
        # MapperBase::setMinMaxCoords (MapperBase.cpp:92-122)
        if not volume.hasMinMaxObjectCoords():
            volume.updateMinMaxCoords()
        self.setMinMaxObjectCoords(volume.minObjectCoord(), volume.maxObjectCoord())
        self.setMinMaxExternalCoords(volume.minExternalCoord(), volume.maxExternalCoord())
        self._polygon_type = PolygonObject.Triangle
        if self._duplication:
            self._normal_type = PolygonObject.PolygonNormal
        self._color_type = PolygonObject.PolygonColor

        nx, ny, nz = volume.resolution()
        mode = (_abi.MODE_SHARED_VERTEX_NORMAL if self.normalType() == PolygonObject.VertexNormal
                else (_abi.MODE_DUP_POLYGON_NORMAL if self._duplication else _abi.MODE_SHARED_POLYGON_NORMAL))
        mn, mx = volume.minObjectCoord(), volume.maxObjectCoord()
        f32 = np.float32
        with np.errstate(divide="ignore", invalid="ignore"):
            scale = [f32(f32(mx[k] - mn[k]) / f32(n - 1)) for k, n in enumerate((nx, ny, nz))]
        params = _abi.make_params(self._isolevel, mode,
                                  (volume.minValue(), volume.maxValue()) if volume.hasMinMaxValues() else None,
                                  mn, scale)
        ctx = self._ctx or default_context()
        coords, normals, conn, sizes = _abi.marching_cubes_host(ctx, volume.volume_array(), params)
        self.sizes = sizes
        # MapperBase::setRange (MapperBase.cpp:54-83): the volume's min/max
        # cache is filled (here by the device scan), then the TF range.
        if not volume.hasMinMaxValues():
            volume.setMinMaxValues(sizes["min_value"], sizes["max_value"])
        set_mapper_range(self._tfunc, code, volume.minValue(), volume.maxValue())
        if not sizes["extracted"] or coords.size == 0:
            return
        self._coords = coords
        self._normals = normals
        if mode != _abi.MODE_DUP_POLYGON_NORMAL:
            self._connections = conn
        self._colors = self._tfunc.color_at(self._isolevel)
        self._opacities = np.array([255], np.uint8)
