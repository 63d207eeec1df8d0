"""kvs::UnstructuredVolumeObject and the unstructured marching mappers, with
the per-cell work on the GPU.

Mirrors (Source/Core/Visualization/):
  UnstructuredVolumeObject  Object/UnstructuredVolumeObject.h:23-120 (input)
  MarchingTetrahedra        Mapper/MarchingTetrahedra.h / .cpp
  MarchingHexahedra         Mapper/MarchingHexahedra.h / .cpp
  MarchingPyramid           Mapper/MarchingPyramid.h / .cpp
  MarchingPrism             Mapper/MarchingPrism.h / .cpp

The constructor form (volume, isolevel, normal_type, duplication,
transfer_function) runs exec at once, like the reference.  The checks and
their messages, the volume's min/max cache (filled by the device scan over
the cells' nodes, GetMinMaxValues' rules), the bounding box
(updateMinMaxCoords), the transfer-function range (MapperBase::setRange) and
the single polygon colour (ColorMap::at(isolevel)) are decided here as the
reference decides them; classification, interpolation, normals and the
compaction in cell order run in libkvsmc's CUDA kernels
(kvsmc_marching_cells_host).  There is no CPU fallback.

Reference behaviour kept:
  * isSuccess() is never set true by these mappers (only their checks set it
    false, MapperBase's initial value is false);
  * with duplication == False (or VertexNormal, which forces it) nothing is
    extracted: the shared-vertex branches are not implemented in the
    reference (MarchingTetrahedra.cpp:244-300; MarchingHexahedra.cpp:135-138
    and the same lines of MarchingPyramid.cpp and MarchingPrism.cpp call only
    the duplicated branch);
  * MarchingHexahedra / Pyramid / Prism set the triangle / polygon-colour /
    polygon-normal types even then, MarchingTetrahedra only with duplication.
"""
import numpy as np

from . import _abi
from .marching_cubes import (ObjectBase, PolygonObject, TransferFunction, _equal, default_context, message_error,
                             set_mapper_range)


class UnstructuredVolumeObject(ObjectBase):
    """kvs::UnstructuredVolumeObject (cell type, nodes, cells, coords,
    connections, values, veclen, min/max cache)."""

    (UnknownCellType, Tetrahedra, Hexahedra, QuadraticTetrahedra, QuadraticHexahedra, Pyramid, Point,
     Prism) = range(8)
    # NumberOfCellNodes (UnstructuredVolumeObject.cpp:27-37)
    _CELL_NODES = (0, 4, 8, 10, 20, 5, 1, 6)

    def __init__(self, cell_type=0, nnodes=0, ncells=0, veclen=1, coords=None, connections=None, values=None):
        super().__init__()
        self._cell_type = int(cell_type)
        self._nnodes = int(nnodes)
        self._ncells = int(ncells)
        self._veclen = int(veclen)
        self._coords = np.zeros(0, np.float32) if coords is None else np.ascontiguousarray(coords, np.float32).reshape(-1)
        self._connections = (np.zeros(0, np.uint32) if connections is None
                             else np.ascontiguousarray(connections, np.uint32).reshape(-1))
        self._values = np.zeros(0, np.float32) if values is None else np.ascontiguousarray(values).reshape(-1)
        self._has_minmax = False
        self._min_value = 0.0
        self._max_value = 0.0

    def setCellType(self, t):
        self._cell_type = int(t)

    def setCellTypeToTetrahedra(self):
        self.setCellType(self.Tetrahedra)

    def setCellTypeToHexahedra(self):
        self.setCellType(self.Hexahedra)

    def setCellTypeToPyramid(self):
        self.setCellType(self.Pyramid)

    def setCellTypeToPrism(self):
        self.setCellType(self.Prism)

    def setNumberOfNodes(self, n):
        self._nnodes = int(n)

    def setNumberOfCells(self, n):
        self._ncells = int(n)

    def setVeclen(self, veclen):
        self._veclen = int(veclen)

    def setCoords(self, coords):
        self._coords = np.ascontiguousarray(coords, np.float32).reshape(-1)

    def setConnections(self, connections):
        self._connections = np.ascontiguousarray(connections, np.uint32).reshape(-1)

    def setValues(self, values):
        self._values = np.ascontiguousarray(values).reshape(-1)
        self._has_minmax = False

    def setMinMaxValues(self, mn, mx):
        self._min_value, self._max_value = float(mn), float(mx)
        self._has_minmax = True

    def cellType(self):
        return self._cell_type

    def numberOfNodes(self):
        return self._nnodes

    def numberOfCells(self):
        return self._ncells

    def numberOfCellNodes(self):
        return self._CELL_NODES[self._cell_type]

    def veclen(self):
        return self._veclen

    def coords(self):
        return self._coords

    def connections(self):
        return self._connections

    def values(self):
        return self._values

    def hasMinMaxValues(self):
        return self._has_minmax

    def minValue(self):
        return self._min_value

    def maxValue(self):
        return self._max_value

    def updateMinMaxCoords(self):
        """UnstructuredVolumeObject::updateMinMaxCoords (UnstructuredVolumeObject.cpp:396-466):
        per axis Math::Min(current, x) / Math::Max(current, x) from the first
        connected node over every connection (over the nodes when there are
        none); a NaN x is taken and the next value replaces it, ties keep the
        later value."""
        if self._coords.size == 0:
            return
        xyz = self._coords.reshape(-1, 3)
        conn = self._connections[:self._ncells * self.numberOfCellNodes()].astype(np.int64)
        seq = xyz if conn.size == 0 else xyz[np.concatenate([conn[:1], conn])]
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        for ax in range(3):
            s = seq[:, ax]
            nan = np.flatnonzero(np.isnan(s))
            if nan.size and nan[-1] == s.size - 1:
                lo[ax] = hi[ax] = s[-1]
                continue
            t = s[nan[-1] + 1:] if nan.size else s
            lo[ax] = t[np.flatnonzero(t == t.min())[-1]]
            hi[ax] = t[np.flatnonzero(t == t.max())[-1]]
        self.setMinMaxObjectCoords(lo, hi)
        if not self.hasMinMaxExternalCoords():
            self.setMinMaxExternalCoords(lo, hi)


def set_bounds_on_device(ctx, volume, abi_cell, connections):
    """UnstructuredVolumeObject::updateMinMaxCoords by kvsmc_cells_bounds."""
    if volume.coords().size == 0:
        return
    lo, hi = _abi.cells_bounds(ctx, abi_cell, volume.coords()[:3 * volume.numberOfNodes()], connections)
    volume.setMinMaxObjectCoords(lo, hi)
    if not volume.hasMinMaxExternalCoords():
        volume.setMinMaxExternalCoords(lo, hi)


class _MarchingCells(PolygonObject):
    """Shared body of the four unstructured marching mappers."""

    CELL = None            # UnstructuredVolumeObject cell type
    ABI_CELL = None        # kvsmc_cell_type
    TYPE_MESSAGE = None    # the mapper's "not <type>-cell data" message
    DTYPE_MESSAGE = "Unsupported data type '{}' of the volume."
    TYPES_NEED_DUPLICATION = False

    def __init__(self, volume=None, isolevel=0.0, normal_type=PolygonObject.PolygonNormal, duplication=True,
                 transfer_function=None, context=None):
        super().__init__()
        self._tfunc = (transfer_function or TransferFunction(256)).copy()
        self._isolevel = float(isolevel)
        self._duplication = bool(duplication)
        self._success = False        # MapperBase() (MapperBase.cpp:23)
        self._ctx = context
        self.sizes = None
        self.setNormalType(normal_type)
        if volume is not None:
            self.exec(volume)

    # MapperBase (Mapper/MapperBase.h:26-63)
    def setIsolevel(self, isolevel):
        self._isolevel = float(isolevel)

    def isolevel(self):
        return self._isolevel

    def setTransferFunction(self, tfunc):
        self._tfunc = tfunc.copy()

    def transferFunction(self):
        return self._tfunc

    def isSuccess(self):
        return self._success

    def isFailure(self):
        return not self._success

    def exec(self, obj):
        """<Mapper>::exec (e.g. MarchingTetrahedra.cpp:46-86)."""
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, UnstructuredVolumeObject):
            self._success = False
            message_error("Input object is not unstructured volume object.")
            return None
        if obj.veclen() != 1:
            self._success = False
            message_error("Input volume is not sclar field data.")
            return None
        if obj.cellType() != self.CELL:
            self._success = False
            message_error(self.TYPE_MESSAGE)
            return None
        if self.normalType() == PolygonObject.VertexNormal:
            self._duplication = False
        try:
            self._mapping(obj)
        except _abi.KvsmcError as e:
            # no CPU fallback: the GPU call failed, so the mapper failed
            self._success = False
            message_error(f"libkvsmc: {e}")
            return None
        return self

    def _mapping(self, volume):
        """<Mapper>::mapping (e.g. MarchingTetrahedra.cpp:94-136)."""
        values = volume.values()
        try:
            code = _abi.dtype_code(values.dtype)
        except TypeError:
            code = None
        npc = volume.numberOfCellNodes()
        ncells = volume.numberOfCells()
        conn = volume.connections()
        if conn.size < ncells * npc or volume.coords().size < 3 * volume.numberOfNodes() \
                or values.size < volume.numberOfNodes():
            raise ValueError("the volume's arrays are shorter than its node / cell counts")
        conn = conn[:ncells * npc]
        ctx = self._ctx or default_context()
        # MapperBase::setRange: min/max cache first (the device scan), then the
        # transfer function's range (MapperBase.cpp:54-83)
        coords = normals = None
        sizes = None
        extract = code is not None and self._duplication
        if code is not None and (extract or not volume.hasMinMaxValues()):
            nodes = volume.numberOfNodes()
            # without extraction only the min/max is wanted: at isolevel NaN no
            # node is above, so only the scan and an empty count pass run
            coords, normals, sizes = _abi.marching_cells_host(
                ctx, self.ABI_CELL, values[:nodes], volume.coords()[:3 * nodes], conn,
                self._isolevel if extract else float("nan"),
                (volume.minValue(), volume.maxValue()) if volume.hasMinMaxValues() else None)
            if not volume.hasMinMaxValues():
                volume.setMinMaxValues(sizes["min_value"], sizes["max_value"])
        self.sizes = sizes
        set_mapper_range(self._tfunc, code, volume.minValue(), volume.maxValue())
        # MapperBase::setMinMaxCoords (MapperBase.cpp:92-122), the volume's
        # updateMinMaxCoords fold run on the GPU
        if not volume.hasMinMaxObjectCoords():
            set_bounds_on_device(ctx, volume, self.ABI_CELL, conn)
        self.setMinMaxObjectCoords(volume.minObjectCoord(), volume.maxObjectCoord())
        self.setMinMaxExternalCoords(volume.minExternalCoord(), volume.maxExternalCoord())
        if not self.TYPES_NEED_DUPLICATION or self._duplication:
            self._polygon_type = PolygonObject.Triangle
            self._color_type = PolygonObject.PolygonColor
            self._normal_type = PolygonObject.PolygonNormal
        if _equal(volume.minValue(), volume.maxValue()):
            return
        if code is None:
            self._success = False
            message_error(self.DTYPE_MESSAGE.format(values.dtype))
            return
        if not extract or coords is None or coords.size == 0:
            return
        self._coords = coords
        self._normals = normals
        self._colors = self._tfunc.color_at(self._isolevel)
        self._opacities = np.array([255], np.uint8)


class MarchingTetrahedra(_MarchingCells):
    """kvs::MarchingTetrahedra (drop-in; per-cell work on the GPU)."""
    CELL = UnstructuredVolumeObject.Tetrahedra
    ABI_CELL = 0
    TYPE_MESSAGE = "Input volume is not tetrahedra-cell data."
    DTYPE_MESSAGE = "Unsupported data type '{}'."
    TYPES_NEED_DUPLICATION = True


class MarchingHexahedra(_MarchingCells):
    """kvs::MarchingHexahedra (drop-in; per-cell work on the GPU)."""
    CELL = UnstructuredVolumeObject.Hexahedra
    ABI_CELL = 1
    TYPE_MESSAGE = "Input volume is not hexhedra-cell data."


class MarchingPyramid(_MarchingCells):
    """kvs::MarchingPyramid (drop-in; per-cell work on the GPU)."""
    CELL = UnstructuredVolumeObject.Pyramid
    ABI_CELL = 2
    TYPE_MESSAGE = "Input volume is not pyramid-cell data."


class MarchingPrism(_MarchingCells):
    """kvs::MarchingPrism (drop-in; per-cell work on the GPU)."""
    CELL = UnstructuredVolumeObject.Prism
    ABI_CELL = 3
    TYPE_MESSAGE = "Input volume is not prism-cell data."


MAPPERS = {UnstructuredVolumeObject.Tetrahedra: MarchingTetrahedra,
           UnstructuredVolumeObject.Hexahedra: MarchingHexahedra,
           UnstructuredVolumeObject.Pyramid: MarchingPyramid,
           UnstructuredVolumeObject.Prism: MarchingPrism}
MAPPERS_BY_ABI = {m.ABI_CELL: m for m in MAPPERS.values()}
