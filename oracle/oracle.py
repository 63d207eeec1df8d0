"""ctypes binding to the C restatement of kvs::MarchingCubes (oracle/mc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline leg.  The product (kvs_gb300) never
imports it.  `build()` compiles the C file with gcc -O3 -ffp-contract=off into
oracle/_build/ (git-ignored), on whichever host runs it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mc_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmc_oracle.so")

DTYPES = [np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16,
          np.uint32, np.uint64, np.float32, np.float64]

MODE_DUP_POLYGON = 0       # duplicated vertices, polygon normals
MODE_SHARED_POLYGON = 1    # shared vertices + connections, polygon normals
MODE_SHARED_VERTEX = 2     # shared vertices + connections, vertex normals


def dtype_code(dt):
    dt = np.dtype(dt)
    for i, d in enumerate(DTYPES):
        if np.dtype(d) == dt:
            return i
    raise ValueError(f"unsupported dtype {dt}")


class _Out(C.Structure):
    _fields_ = [
        ("success", C.c_int), ("extracted", C.c_int),
        ("coords", C.POINTER(C.c_float)), ("ncoords", C.c_uint64),
        ("normals", C.POINTER(C.c_float)), ("nnormals", C.c_uint64),
        ("connections", C.POINTER(C.c_uint32)), ("nconnections", C.c_uint64),
        ("color", C.c_ubyte * 3),
        ("vmin", C.c_double), ("vmax", C.c_double),
        ("min_obj", C.c_float * 3), ("max_obj", C.c_float * 3),
        ("seconds", C.c_double),
    ]


_lib = None


def build(force=False):
    """Compile mc_oracle.c.  Cheap (one C file); rebuilt when the source is newer."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
           "-D_POSIX_C_SOURCE=199309L", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.mco_minmax.argtypes = [C.c_int, C.c_void_p, C.c_uint64,
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.mco_extract.argtypes = [C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                     C.c_double, C.c_int, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.POINTER(_Out)]
        _lib.mco_marching_cubes.argtypes = [
            C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
            C.c_double, C.c_int, C.c_int,
            C.c_int, C.c_double, C.c_double,
            C.c_int, C.c_void_p,
            C.c_int, C.c_void_p, C.c_void_p,
            C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float,
            C.POINTER(_Out)]
        _lib.mco_color_at.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_void_p]
        _lib.mco_free.argtypes = [C.POINTER(_Out)]
        _lib.mco_dup_checksum.argtypes = [C.c_int, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                          C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                          C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                          C.c_uint64, C.POINTER(C.c_uint64)]
    return _lib


def _arr(ptr, n, dt):
    if n == 0:
        return np.zeros(0, dtype=dt)
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def _collect(o):
    return dict(
        success=bool(o.success), extracted=bool(o.extracted),
        coords=_arr(o.coords, o.ncoords, np.float32),
        normals=_arr(o.normals, o.nnormals, np.float32),
        connections=_arr(o.connections, o.nconnections, np.uint32),
        color=np.array(o.color[:], np.uint8),
        vol_min=o.vmin, vol_max=o.vmax,
        min_obj=np.array(o.min_obj[:], np.float32), max_obj=np.array(o.max_obj[:], np.float32),
        seconds=o.seconds)


def minmax(values):
    v = np.ascontiguousarray(values)
    mn, mx = C.c_double(), C.c_double()
    if lib().mco_minmax(dtype_code(v.dtype), v.ctypes.data, v.size, C.byref(mn), C.byref(mx)):
        raise ValueError("empty volume")
    return mn.value, mx.value


def extract(values, isolevel, mode, vmin, vmax, min_coord=(0, 0, 0), scale=(1, 1, 1)):
    """One extraction with min/max, bbox and scale already decided."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    mc = np.asarray(min_coord, np.float32)
    sc = np.asarray(scale, np.float32)
    o = _Out()
    rc = lib().mco_extract(dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel), int(mode),
                           float(vmin), float(vmax), mc.ctypes.data, sc.ctypes.data, C.byref(o))
    if rc:
        raise MemoryError("oracle extraction failed")
    r = _collect(o)
    lib().mco_free(C.byref(o))
    return r


def marching_cubes(values, isolevel, normal_type="polygon", duplication=True, minmax=None,
                   rect_coords=None, obj_coords=None, colormap=None, tf_range=None):
    """The whole constructor/exec flow; colormap = (resolution, 3) uint8 table or None."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    rc = np.ascontiguousarray(rect_coords, dtype=np.float32) if rect_coords is not None else None
    mn = mx = None
    if obj_coords is not None:
        mn = np.ascontiguousarray(obj_coords[0], dtype=np.float32)
        mx = np.ascontiguousarray(obj_coords[1], dtype=np.float32)
    cm = np.ascontiguousarray(colormap, dtype=np.uint8) if colormap is not None else None
    o = _Out()
    st = lib().mco_marching_cubes(
        dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, float(isolevel),
        0 if normal_type == "vertex" else 1, 1 if duplication else 0,
        1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0,
        float(minmax[1]) if minmax is not None else 0.0,
        1 if rc is not None else 0, rc.ctypes.data if rc is not None else None,
        1 if obj_coords is not None else 0,
        mn.ctypes.data if mn is not None else None, mx.ctypes.data if mx is not None else None,
        cm.ctypes.data if cm is not None else None, cm.shape[0] if cm is not None else 0,
        1 if tf_range is not None else 0,
        float(tf_range[0]) if tf_range is not None else 0.0,
        float(tf_range[1]) if tf_range is not None else 0.0,
        C.byref(o))
    if st:
        raise RuntimeError(f"oracle marching_cubes failed ({st})")
    r = _collect(o)
    lib().mco_free(C.byref(o))
    return r


def mix_checksum(words, chunk_words):
    """The checksum of kvsmc_checksum_words in numpy (per chunk of a uint32
    array, index from the array's start); a check of the C and CUDA sums."""
    w = np.ascontiguousarray(words).view(np.uint32).astype(np.uint64)
    i = np.arange(w.size, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = (i * np.uint64(0x9E3779B97F4A7C15)) ^ (w * np.uint64(0xC2B2AE3D27D4EB4F))
        x ^= x >> np.uint64(31)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(29)
    n = (w.size + chunk_words - 1) // chunk_words
    return np.array([int(x[c * chunk_words:(c + 1) * chunk_words].sum(dtype=np.uint64)) for c in range(n)],
                    dtype=np.uint64)


def dup_checksum(values, isolevel, vmin, vmax, z0=0, z1=None, min_coord=(0, 0, 0), scale=(1, 1, 1),
                 chunk_tris=1 << 20, nchunks=None):
    """Duplicated-mode extraction over the cell planes [z0, z1) of the whole
    volume, folded into per-chunk checksums (mco_dup_checksum).  Returns
    (triangles, coord sums, normal sums); the sums cover chunks of chunk_tris
    triangles, 9 words (coords) and 3 words (normals) per triangle.  The C
    call releases the GIL, so threads can run several isolevels at once."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    z1 = nz - 1 if z1 is None else z1
    if nchunks is None:
        # at most 5 triangles per cell
        nchunks = max(1, ((nx - 1) * (ny - 1) * (z1 - z0) * 5 + chunk_tris - 1) // chunk_tris)
    cs = np.zeros(nchunks, np.uint64)
    ns = np.zeros(nchunks, np.uint64)
    mc = np.asarray(min_coord, np.float32)
    sc = np.asarray(scale, np.float32)
    t = C.c_uint64()
    rc = lib().mco_dup_checksum(dtype_code(v.dtype), v.ctypes.data, nx, ny, nz, z0, z1, float(isolevel),
                                float(vmin), float(vmax), mc.ctypes.data, sc.ctypes.data, chunk_tris,
                                cs.ctypes.data, ns.ctypes.data, nchunks, C.byref(t))
    if rc:
        raise RuntimeError(f"oracle checksum failed ({rc})")
    used = max(1, (t.value + chunk_tris - 1) // chunk_tris)
    return t.value, cs[:used], ns[:used]
