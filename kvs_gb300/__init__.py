"""kvs_gb300: GB300-native structured-grid marching cubes (kvs::cuda::MarchingCubes).

The compute path is libkvsmc.so (hand-written CUDA for sm_103a behind the C ABI
in include/kvsmc.h).  This package holds the Python host layer over that ABI.
"""
from . import _abi  # noqa: F401
from .marching_cubes import (MarchingCubes, PolygonObject, StructuredVolumeObject,  # noqa: F401
                             TransferFunction, default_context)
from .marching_cells import (MarchingHexahedra, MarchingPrism, MarchingPyramid,  # noqa: F401
                             MarchingTetrahedra, UnstructuredVolumeObject)

__all__ = ["MarchingCubes", "PolygonObject", "StructuredVolumeObject", "TransferFunction",
           "default_context", "UnstructuredVolumeObject", "MarchingTetrahedra", "MarchingHexahedra",
           "MarchingPyramid", "MarchingPrism"]
