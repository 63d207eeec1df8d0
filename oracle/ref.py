"""ctypes binding to the reference kvs::MarchingCubes and kvs::Isosurface built by
oracle/Makefile.ref.

Test infrastructure only (parity anchor).  The library exists only where the
reference sources were available to compile it; `available()` says whether it
was built.  Runs Source/Core/Visualization/Mapper/MarchingCubes.cpp:25-37
(constructor -> exec -> mapping) on a StructuredVolumeObject made from a
numpy array and returns the PolygonObject's arrays.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libkvsref_mc.so")
# The reference tree this recipe compiles: $KVS_SRC, else the location the
# build container mounts it at.  Every other file takes the path from here.
REFERENCE_SOURCE = os.environ.get("KVS_SRC") or "/root/reference/Source"

# dtype codes: order of the reference's type switch (MarchingCubes.cpp:115-124)
DTYPES = [np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16,
          np.uint32, np.uint64, np.float32, np.float64]


def dtype_code(dt):
    dt = np.dtype(dt)
    for i, d in enumerate(DTYPES):
        if np.dtype(d) == dt:
            return i
    raise ValueError(f"unsupported dtype {dt}")


class _Result(C.Structure):
    _fields_ = [
        ("success", C.c_int),
        ("ncoords", C.c_ulonglong), ("nnormals", C.c_ulonglong),
        ("nconnections", C.c_ulonglong), ("ncolors", C.c_ulonglong),
        ("nopacities", C.c_ulonglong),
        ("coords", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
        ("connections", C.POINTER(C.c_uint)), ("colors", C.POINTER(C.c_ubyte)),
        ("opacities", C.POINTER(C.c_ubyte)),
        ("polygon_type", C.c_int), ("normal_type", C.c_int), ("color_type", C.c_int),
        ("vol_has_minmax", C.c_int), ("vol_min", C.c_double), ("vol_max", C.c_double),
        ("min_obj", C.c_float * 3), ("max_obj", C.c_float * 3),
        ("min_ext", C.c_float * 3), ("max_ext", C.c_float * 3),
        ("seconds", C.c_double),
    ]


_lib = None


def build(jobs=8, quiet=True):
    """Compile the reference path from its sources (only where they exist)."""
    if not os.path.isdir(REFERENCE_SOURCE):
        return False
    cmd = ["make", "-f", os.path.join(HERE, "Makefile.ref"), f"KVS_SRC={REFERENCE_SOURCE}",
           f"-j{jobs}"]
    out = subprocess.run(cmd, cwd=os.path.dirname(HERE), capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + (out.stderr or "")[-4000:])
    return True


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(LIB_PATH)
        _lib.kvsref_marching_cubes.restype = C.c_int
        _lib.kvsref_marching_cubes.argtypes = [
            C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
            C.c_double, C.c_int, C.c_int,
            C.c_int, C.c_double, C.c_double,
            C.c_int, C.c_void_p,
            C.c_int, C.c_void_p, C.c_void_p,
            C.c_int, C.c_int, C.c_float, C.c_float,
            C.c_int, C.POINTER(_Result)]
        _lib.kvsref_isosurface.restype = C.c_int
        _lib.kvsref_isosurface.argtypes = [
            C.c_int, C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint,
            C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
            C.c_int, C.c_int, C.c_float, C.c_float, C.POINTER(_Result)]
        _lib.kvsref_slice_plane.restype = C.c_int
        _lib.kvsref_slice_plane.argtypes = [
            C.c_int, C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_void_p,
            C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_float, C.c_float,
            C.c_int, C.c_void_p, C.c_void_p, C.POINTER(_Result)]
        _lib.kvsref_marching_cubes_export.restype = C.c_int
        _lib.kvsref_marching_cubes_export.argtypes = [
            C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_int, C.c_int, C.c_int, C.c_char_p]
        _lib.kvsref_marching_cubes_stl.restype = C.c_int
        _lib.kvsref_marching_cubes_stl.argtypes = [
            C.c_int, C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_double, C.c_int, C.c_int, C.c_char_p]
        _lib.kvsref_marching_cells.restype = C.c_int
        _lib.kvsref_marching_cells.argtypes = [
            C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_ulonglong,
            C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_float,
            C.c_float, C.c_int, C.POINTER(_Result)]
        _lib.kvsref_slice_cells.restype = C.c_int
        _lib.kvsref_slice_cells.argtypes = [
            C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_void_p, C.c_ulonglong,
            C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_float, C.c_float,
            C.POINTER(_Result)]
        _lib.kvsref_write_ply.restype = C.c_int
        _lib.kvsref_write_ply.argtypes = [C.c_void_p, C.c_ulonglong, C.c_void_p, C.c_ulonglong, C.c_void_p,
                                          C.c_ulonglong, C.c_int, C.c_int, C.c_char_p]
        _lib.kvsref_free.argtypes = [C.POINTER(_Result)]
        _lib.kvsref_hydrogen.argtypes = [C.c_uint, C.c_void_p]
        _lib.kvsref_default_colormap.argtypes = [C.c_int, C.c_void_p]
        _lib.kvsref_color_at.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, C.c_void_p]
    return _lib


def _arr(ptr, n, dt):
    if n == 0:
        return np.zeros(0, dtype=dt)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def marching_cubes(values, isolevel, normal_type="polygon", duplication=True,
                   minmax=None, rect_coords=None, obj_coords=None,
                   tf_resolution=256, tf_range=None, repeat=1):
    """values: numpy array shaped (nz, ny, nx) (x fastest, like KVS)."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    r = _Result()
    rc = np.ascontiguousarray(rect_coords, dtype=np.float32) if rect_coords is not None else None
    mn = mx = None
    if obj_coords is not None:
        mn = np.ascontiguousarray(obj_coords[0], dtype=np.float32)
        mx = np.ascontiguousarray(obj_coords[1], dtype=np.float32)
    st = lib().kvsref_marching_cubes(
        dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel),
        0 if normal_type == "polygon" else 1, 1 if duplication else 0,
        1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        1 if rc is not None else 0, rc.ctypes.data if rc is not None else None,
        1 if obj_coords is not None else 0,
        mn.ctypes.data if mn is not None else None,
        mx.ctypes.data if mx is not None else None,
        tf_resolution, 1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0,
        repeat, C.byref(r))
    if st != 0:
        raise RuntimeError("kvsref_marching_cubes failed")
    out = dict(
        success=bool(r.success),
        coords=_arr(r.coords, r.ncoords, np.float32),
        normals=_arr(r.normals, r.nnormals, np.float32),
        connections=_arr(r.connections, r.nconnections, np.uint32),
        colors=_arr(r.colors, r.ncolors, np.uint8),
        opacities=_arr(r.opacities, r.nopacities, np.uint8),
        polygon_type=r.polygon_type, normal_type=r.normal_type, color_type=r.color_type,
        vol_has_minmax=bool(r.vol_has_minmax), vol_min=r.vol_min, vol_max=r.vol_max,
        min_obj=np.array(r.min_obj[:], np.float32), max_obj=np.array(r.max_obj[:], np.float32),
        min_ext=np.array(r.min_ext[:], np.float32), max_ext=np.array(r.max_ext[:], np.float32),
        seconds=r.seconds)
    lib().kvsref_free(C.byref(r))
    return out


def _collect(r):
    out = dict(
        success=bool(r.success),
        coords=_arr(r.coords, r.ncoords, np.float32),
        normals=_arr(r.normals, r.nnormals, np.float32),
        connections=_arr(r.connections, r.nconnections, np.uint32),
        colors=_arr(r.colors, r.ncolors, np.uint8),
        opacities=_arr(r.opacities, r.nopacities, np.uint8),
        polygon_type=r.polygon_type, normal_type=r.normal_type, color_type=r.color_type,
        vol_has_minmax=bool(r.vol_has_minmax), vol_min=r.vol_min, vol_max=r.vol_max,
        min_obj=np.array(r.min_obj[:], np.float32), max_obj=np.array(r.max_obj[:], np.float32),
        min_ext=np.array(r.min_ext[:], np.float32), max_ext=np.array(r.max_ext[:], np.float32))
    lib().kvsref_free(C.byref(r))
    return out


def isosurface(values, form, isolevel=0.0, normal_type="polygon", duplication=True, minmax=None,
               tf_resolution=256, tf_range=None):
    """The reference kvs::Isosurface through constructor `form` (0: volume,
    normal type -- isolevel from the min/max; 1: + isolevel; 2: + duplication
    and transfer function) on a uniform volume shaped (nz, ny, nx)."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    r = _Result()
    st = lib().kvsref_isosurface(
        int(form), dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel),
        0 if normal_type == "polygon" else 1, 1 if duplication else 0,
        1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        tf_resolution, 1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0, C.byref(r))
    if st != 0:
        raise RuntimeError("kvsref_isosurface failed")
    return _collect(r)


CELL_NODES = {0: 4, 1: 8, 2: 5, 3: 6}   # tetrahedra, hexahedra, pyramid, prism


def marching_cells(cell_type, values, coords, connections, isolevel, form=0, normal_type="polygon",
                   duplication=True, minmax=None, tf_resolution=256, tf_range=None, repeat=1):
    """The reference unstructured marching mapper of `cell_type` (0 tetrahedra,
    1 hexahedra, 2 pyramid, 3 prism) -- form 0 -- or kvs::Isosurface routing to
    it -- form 1 -- on an UnstructuredVolumeObject of nnodes values, float32
    coords (3 per node) and uint32 connections (nodes per cell x ncells)."""
    v = np.ascontiguousarray(values).reshape(-1)
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(connections, np.uint32).reshape(-1)
    npc = CELL_NODES[int(cell_type)]
    if c.size != 3 * v.size or k.size % npc:
        raise ValueError("coords / connections do not match the node count / cell type")
    r = _Result()
    st = lib().kvsref_marching_cells(
        int(form), int(cell_type), dtype_code(v.dtype), v.ctypes.data, v.size, c.ctypes.data, k.ctypes.data,
        k.size // npc, float(isolevel), 0 if normal_type == "polygon" else 1, 1 if duplication else 0,
        1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        tf_resolution, 1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0, int(repeat), C.byref(r))
    if st != 0:
        raise RuntimeError("kvsref_marching_cells failed")
    seconds = r.seconds
    out = _collect(r)
    out["seconds"] = seconds
    return out


def slice_cells(cell_type, values, coords, connections, coefficients=None, point=None, normal=None, minmax=None,
                tf_resolution=256, tf_range=None):
    """The reference kvs::SlicePlane on an UnstructuredVolumeObject (cell types
    as marching_cells), by plane coefficients or by a point and a normal."""
    v = np.ascontiguousarray(values).reshape(-1)
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(connections, np.uint32).reshape(-1)
    npc = CELL_NODES[int(cell_type)]
    if coefficients is not None:
        form, plane = 0, np.ascontiguousarray(coefficients, np.float32)
    else:
        form, plane = 1, np.ascontiguousarray(list(point) + list(normal), np.float32)
    r = _Result()
    st = lib().kvsref_slice_cells(
        form, int(cell_type), dtype_code(v.dtype), v.ctypes.data, v.size, c.ctypes.data, k.ctypes.data,
        k.size // npc, plane.ctypes.data, 1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        tf_resolution, 1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0, C.byref(r))
    if st != 0:
        raise RuntimeError("kvsref_slice_cells failed")
    return _collect(r)


def slice_plane(values, coefficients=None, point=None, normal=None, minmax=None, tf_resolution=256,
                tf_range=None, obj_coords=None):
    """The reference kvs::SlicePlane on a uniform volume shaped (nz, ny, nx):
    by plane coefficients (a, b, c, d), or by a point and a normal;
    obj_coords = (min xyz, max xyz) presets the volume's object coords."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    if coefficients is not None:
        form, plane = 0, np.ascontiguousarray(coefficients, np.float32)
    else:
        form, plane = 1, np.ascontiguousarray(list(point) + list(normal), np.float32)
    if obj_coords is not None:
        lo, hi = (np.ascontiguousarray(c, np.float32) for c in obj_coords)
    r = _Result()
    st = lib().kvsref_slice_plane(
        form, dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, plane.ctypes.data,
        1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        tf_resolution, 1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0,
        1 if obj_coords is not None else 0,
        lo.ctypes.data if obj_coords is not None else None,
        hi.ctypes.data if obj_coords is not None else None, C.byref(r))
    if st != 0:
        raise RuntimeError("kvsref_slice_plane failed")
    return _collect(r)


def marching_cubes_stl(values, isolevel, normal_type="polygon", duplication=True, path=None):
    """The reference MarchingCubes result exported by PolygonExporter<kvs::Stl>
    as a binary STL file; returns the file's bytes."""
    import tempfile
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    own = path is None
    if own:
        fd, path = tempfile.mkstemp(suffix=".stl")
        os.close(fd)
    try:
        st = lib().kvsref_marching_cubes_stl(dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel),
                                             0 if normal_type == "polygon" else 1, 1 if duplication else 0,
                                             path.encode())
        if st != 0:
            raise RuntimeError(f"kvsref_marching_cubes_stl failed ({st})")
        with open(path, "rb") as f:
            return f.read()
    finally:
        if own:
            os.remove(path)


EXPORT_FORMATS = {"stl_binary": 0, "stl_ascii": 1, "kvsml_ascii": 2, "kvsml_external_ascii": 3,
                  "kvsml_external_binary": 4}


def marching_cubes_export(values, isolevel, normal_type, duplication, fmt, path):
    """The reference MarchingCubes result written by the reference's STL or
    KVSML polygon writer (EXPORT_FORMATS) to `path` (KVSML external data files
    beside it)."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    st = lib().kvsref_marching_cubes_export(dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel),
                                            0 if normal_type == "polygon" else 1, 1 if duplication else 0,
                                            EXPORT_FORMATS[fmt], path.encode())
    if st != 0:
        raise RuntimeError(f"kvsref_marching_cubes_export failed ({st})")


def hydrogen(res):
    out = np.zeros((res, res, res), np.uint8)
    if lib().kvsref_hydrogen(res, out.ctypes.data) != 0:
        raise RuntimeError("hydrogen failed")
    return out


def default_colormap(resolution=256):
    t = np.zeros(resolution * 3, np.uint8)
    n = lib().kvsref_default_colormap(resolution, t.ctypes.data)
    return t[:n].reshape(-1, 3)


def color_at(resolution, tf_min, tf_max, value):
    rgb = np.zeros(3, np.uint8)
    lib().kvsref_color_at(resolution, tf_min, tf_max, value, rgb.ctypes.data)
    return rgb


def write_ply(path, coords, colors, normals, color_type="polygon", normal_type="polygon"):
    """The reference PolygonExporter<kvs::Ply> + Ply::write (Binary) of a
    connection-less triangle mesh; returns the file's bytes."""
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(colors, np.uint8).reshape(-1)
    n = np.ascontiguousarray(normals, np.float32).reshape(-1)
    st = lib().kvsref_write_ply(c.ctypes.data, c.size, k.ctypes.data if k.size else None, k.size,
                                n.ctypes.data if n.size else None, n.size, 0 if color_type == "vertex" else 1,
                                0 if normal_type == "vertex" else 1, str(path).encode())
    if st != 0:
        raise RuntimeError(f"kvsref_write_ply failed ({st})")
    return open(path, "rb").read()
