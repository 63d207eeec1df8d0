"""kvs::Isosurface with its structured-grid branch on the GPU.

Mirrors the reference mapper (Source/Core/Visualization/Mapper/Isosurface.h:23-57,
Isosurface.cpp): the same three constructor forms, the same exec/mapping
checks and messages, and for a structured volume the same result as the
reference, which builds a kvs::MarchingCubes and shallow-copies its arrays
(Isosurface.cpp:176-191); here that mapper is kvs_gb300's MarchingCubes, so
the per-cell work runs in libkvsmc's CUDA kernels.

    Isosurface(volume, normal_type=PN)               isolevel = (max + min) * 0.5 (Isosurface.cpp:23-40)
    Isosurface(volume, isolevel, normal_type=PN)     (Isosurface.cpp:49-65)
    Isosurface(volume, isolevel, normal_type, duplication, transfer_function)   (Isosurface.cpp:77-96)

As in the reference:
  * VertexNormal forces shared vertices (duplication = False);
  * the volume's min/max cache is filled before the default isolevel is taken
    (here by the device min/max scan, GetMinMaxValues' rules);
  * isSuccess() is never set true by this mapper (the reference leaves
    MapperBase's initial false, MapperBase.cpp:23); only the checks set it
    false.
Unlike the reference, a failure of the GPU mapper is not swallowed: exec
reports "Cannot create isosurfaces." with the cause and returns None (the
reference tests `new` for null and carries on with empty arrays).  An
UnstructuredVolumeObject goes, by its cell type, to this package's
MarchingTetrahedra / MarchingHexahedra / MarchingPyramid / MarchingPrism
(Isosurface.cpp:193-258); other cell types give an empty result, as there.
"""
import numpy as np

from . import _abi
from .marching_cells import MAPPERS, UnstructuredVolumeObject
from .marching_cubes import (MarchingCubes, PolygonObject, StructuredVolumeObject, TransferFunction,
                             default_context, message_error)


class Isosurface(PolygonObject):
    """kvs::Isosurface (drop-in; structured volumes on the GPU)."""

    def __init__(self, volume=None, isolevel=None, normal_type=PolygonObject.PolygonNormal,
                 duplication=True, transfer_function=None, context=None):
        super().__init__()
        self._tfunc = (transfer_function or TransferFunction(256)).copy()
        self._duplication = bool(duplication)
        self._ctx = context
        self._success = False        # MapperBase() (MapperBase.cpp:23)
        self._isolevel = 0.0 if isolevel is None else float(isolevel)
        self.setNormalType(normal_type)
        if volume is None:
            return
        if isolevel is None:
            # Isosurface( volume, normal_type ) (Isosurface.cpp:23-40)
            if not volume.hasMinMaxValues():
                self._update_min_max(volume)
            self._isolevel = (volume.maxValue() + volume.minValue()) * 0.5
        if normal_type == PolygonObject.VertexNormal:
            self._duplication = False
        self.exec(volume)

    def _update_min_max(self, volume):
        """StructuredVolumeObject::updateMinMaxValues (StructuredVolumeObject.cpp:431-450)
        or UnstructuredVolumeObject::updateMinMaxValues (UnstructuredVolumeObject.cpp:469-487)
        by the device scan."""
        ctx = self._ctx or default_context()
        if isinstance(volume, UnstructuredVolumeObject):
            # isolevel NaN: no node is above it, so only the min/max scan and an
            # empty count pass run
            ct = {c: m.ABI_CELL for c, m in MAPPERS.items()}.get(volume.cellType())
            if ct is None:
                raise ValueError("min/max of an unstructured volume needs a marching cell type")
            n = volume.numberOfNodes()
            conn = volume.connections()[:volume.numberOfCells() * volume.numberOfCellNodes()]
            _, _, sizes = _abi.marching_cells_host(ctx, ct, volume.values()[:n], volume.coords()[:3 * n], conn,
                                                   float("nan"))
            volume.setMinMaxValues(sizes["min_value"], sizes["max_value"])
            return
        dv = _abi.DeviceVolume.upload(ctx, volume.volume_array())
        try:
            mn, mx = dv.minmax()
        finally:
            dv.free()
        volume.setMinMaxValues(mn, mx)

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
        """Isosurface::exec (Isosurface.cpp:104-124)."""
        if obj is None:
            self._success = False
            message_error("Input object is NULL.")
            return None
        if not isinstance(obj, (StructuredVolumeObject, UnstructuredVolumeObject)):
            self._success = False
            message_error("Input object is not volume dat.")
            return None
        if not self._mapping(obj):
            return None
        return self

    def _mapping(self, volume):
        """Isosurface::mapping (Isosurface.cpp:142-258)."""
        if volume.veclen() != 1:
            self._success = False
            message_error("Input object is not scalar field dat.")
            return True
        if isinstance(volume, UnstructuredVolumeObject):
            mapper = MAPPERS.get(volume.cellType())
            if mapper is None:
                return True            # default: break (Isosurface.cpp:256)
            mc = mapper(None, self._isolevel, self.normalType(), self._duplication, self._tfunc,
                        context=self._ctx)
            if mc.exec(volume) is None:
                self._success = False
                message_error("Cannot create isosurfaces.")
                return False
        else:
            mc = MarchingCubes(volume, self._isolevel, self.normalType(), self._duplication, self._tfunc,
                               context=self._ctx)
        if isinstance(volume, StructuredVolumeObject) and mc.isFailure():
            self._success = False
            message_error("Cannot create isosurfaces.")
            return False
        # shallow_copy (Isosurface.cpp:152-170)
        self._coords = mc.coords()
        self._colors = mc.colors()
        self._normals = mc.normals()
        self._connections = mc.connections()
        self._opacities = mc.opacities()
        self._polygon_type = mc.polygonType()
        self._color_type = mc.colorType()
        self._normal_type = mc.normalType()
        self.setMinMaxObjectCoords(mc.minObjectCoord(), mc.maxObjectCoord())
        self.setMinMaxExternalCoords(mc.minExternalCoord(), mc.maxExternalCoord())
        self.sizes = mc.sizes
        return True
