"""KVSML structured volumes and AVS fields loaded straight into resident
device volumes (kvsmc_kvsml_read_info / kvsmc_volume_load_kvsml,
kvsmc_avs_read_info / kvsmc_volume_load_avs).

The reference reads a .kvsml file into a host kvs::StructuredVolumeObject
(StructuredVolumeObject::read, Object/StructuredVolumeObject.cpp:171-229);
here the same file becomes a kvsmc volume on the GPU, ready for batches,
plans and the server, with the min/max cache and coordinates the reference
would give the host object.
"""
import ctypes as C

import numpy as np

from . import _abi

FORMATS = ("ascii", "external ascii", "external binary")


def _info_dict(i):
    return {
        "dtype": np.dtype(_abi.DTYPES[i.dtype]) if 0 <= i.dtype < len(_abi.DTYPES) else None,
        "resolution": (i.nx, i.ny, i.nz), "veclen": i.veclen, "uniform": bool(i.grid_uniform),
        "format": FORMATS[i.data_format], "byte_swap": bool(i.byte_swap),
        "min_value": i.min_value if i.has_min_value else None,
        "max_value": i.max_value if i.has_max_value else None,
        "volume_min": i.volume_min, "volume_max": i.volume_max,
        "min_object_coord": np.array(i.min_object_coord[:], np.float32),
        "max_object_coord": np.array(i.max_object_coord[:], np.float32),
        "min_external_coord": np.array(i.min_external_coord[:], np.float32) if i.has_external_coord else None,
        "max_external_coord": np.array(i.max_external_coord[:], np.float32) if i.has_external_coord else None,
    }


def read_info(path):
    """The header of a .kvsml structured volume (no data read)."""
    info = _abi.KvsmlInfo()
    st = _abi.load().kvsmc_kvsml_read_info(str(path).encode(), C.byref(info))
    if st:
        raise _abi.KvsmcError(st, f"kvsml header of {path}: {_abi.status_string(st)}")
    return _info_dict(info)


def read_avs_info(path):
    """The header of an AVS field file (.fld)."""
    info = _abi.KvsmlInfo()
    st = _abi.load().kvsmc_avs_read_info(str(path).encode(), C.byref(info))
    if st:
        raise _abi.KvsmcError(st, f"AVS header of {path}: {_abi.status_string(st)}")
    return _info_dict(info)


def load_avs(ctx, path):
    """(DeviceVolume, info) of a uniform scalar AVS field (.fld)."""
    info = _abi.KvsmlInfo()
    h = C.c_void_p()
    ctx.check(ctx.lib.kvsmc_volume_load_avs(ctx.handle, str(path).encode(), C.byref(h), C.byref(info)),
              "kvsmc_volume_load_avs")
    d = _info_dict(info)
    nx, ny, nz = d["resolution"]
    return _abi.DeviceVolume(ctx, h, d["dtype"], (nz, ny, nx)), d


def load_kvsml(ctx, path):
    """(DeviceVolume, info) of a .kvsml uniform scalar volume."""
    info = _abi.KvsmlInfo()
    h = C.c_void_p()
    ctx.check(ctx.lib.kvsmc_volume_load_kvsml(ctx.handle, str(path).encode(), C.byref(h), C.byref(info)),
              "kvsmc_volume_load_kvsml")
    d = _info_dict(info)
    nx, ny, nz = d["resolution"]
    return _abi.DeviceVolume(ctx, h, d["dtype"], (nz, ny, nx)), d
