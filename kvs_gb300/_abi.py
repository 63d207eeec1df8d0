"""ctypes binding to libkvsmc.so (include/kvsmc.h).

The library is built in-tree by kvs_gb300/build.py.  There is no fallback:
if the shared library is missing, importing this module raises.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libkvsmc.so")

# status codes (kvsmc_status)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED_DTYPE = 2
ERR_OUT_OF_MEMORY = 3
ERR_CUDA = 4
ERR_NO_DEVICE = 5
ERR_CAPACITY = 6
ERR_TOO_LARGE = 7
ERR_TIMEOUT = 8
ERR_BUDGET = 9

# dtype codes (kvsmc_dtype): the reference's type-switch order
DTYPES = [np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16,
          np.uint32, np.uint64, np.float32, np.float64]

MODE_DUP_POLYGON_NORMAL = 0
MODE_SHARED_POLYGON_NORMAL = 1
MODE_SHARED_VERTEX_NORMAL = 2

# Every exported symbol of include/kvsmc.h.
EXPORTS = [
    "kvsmc_create", "kvsmc_destroy", "kvsmc_status_string", "kvsmc_last_error",
    "kvsmc_stream", "kvsmc_set_stream", "kvsmc_synchronize", "kvsmc_kernel_launches",
    "kvsmc_volume_upload", "kvsmc_volume_from_device", "kvsmc_volume_update",
    "kvsmc_volume_free", "kvsmc_volume_minmax",
    "kvsmc_count", "kvsmc_extract_device", "kvsmc_marching_cubes_host",
    "kvsmc_count_batch", "kvsmc_extract_batch", "kvsmc_set_kernel_path",
    "kvsmc_selftest_interpolation", "kvsmc_profile_enable", "kvsmc_profile_read",
    "kvsmc_extract_batch_host", "kvsmc_extract_noalloc",
    "kvsmc_plan_create", "kvsmc_plan_launch", "kvsmc_plan_wait", "kvsmc_plan_kernels", "kvsmc_plan_destroy",
    "kvsmc_server_create", "kvsmc_server_submit", "kvsmc_server_poll", "kvsmc_server_release",
    "kvsmc_server_stats", "kvsmc_server_destroy", "kvsmc_copy_to_host",
    "kvsmc_size_class", "kvsmc_tune_resolve", "kvsmc_tuning_set", "kvsmc_tuning_get",
    "kvsmc_tuning_force", "kvsmc_autotune", "kvsmc_stl_records", "kvsmc_write_stl",
    "kvsmc_write_stl_host", "kvsmc_volume_download", "kvsmc_kvsml_read_info", "kvsmc_volume_load_kvsml",
    "kvsmc_avs_read_info", "kvsmc_volume_load_avs",
    "kvsmc_slice_count", "kvsmc_slice_extract_device", "kvsmc_slice_plane",
    "kvsmc_marching_cells_host", "kvsmc_marching_cells_device", "kvsmc_selftest_cells", "kvsmc_slice_cells_host",
    "kvsmc_cells_bounds", "kvsmc_marching_cells_sweep_device", "kvsmc_ply_record_bytes", "kvsmc_ply_header", "kvsmc_ply_records", "kvsmc_write_ply", "kvsmc_write_ply_host",
    "kvsmc_checksum_words", "kvsmc_set_wait_limit", "kvsmc_write_stl_ascii", "kvsmc_write_stl_ascii_host",
    "kvsmc_write_kvsml_polygon",
]

PATH_AUTO = 0      # streaming kernels where eligible
PATH_GATHER = 1    # gather kernels only


def dtype_code(dt):
    dt = np.dtype(dt)
    for i, d in enumerate(DTYPES):
        if np.dtype(d) == dt:
            return i
    raise TypeError(f"Unsupported data type '{dt}'.")


class Params(C.Structure):
    _fields_ = [("isolevel", C.c_double), ("mode", C.c_int32), ("has_minmax", C.c_int32),
                ("min_value", C.c_double), ("max_value", C.c_double),
                ("min_coord", C.c_float * 3), ("scale", C.c_float * 3)]


class Sizes(C.Structure):
    _fields_ = [("ntriangles", C.c_uint64), ("nvertices", C.c_uint64), ("ncoords", C.c_uint64),
                ("nnormals", C.c_uint64), ("nconnections", C.c_uint64),
                ("min_value", C.c_double), ("max_value", C.c_double),
                ("extracted", C.c_int32), ("reserved", C.c_int32)]


class ServerConfig(C.Structure):
    _fields_ = [("output_budget_bytes", C.c_uint64), ("max_batch", C.c_int32), ("workers", C.c_int32)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int), ("batch_size", C.c_int32), ("sizes", Sizes),
                ("d_coords", C.c_void_p), ("d_normals", C.c_void_p),
                ("submit_s", C.c_double), ("start_s", C.c_double), ("done_s", C.c_double)]


class Request(C.Structure):
    _fields_ = [("volume", C.c_void_p), ("params", Params),
                ("d_coords", C.c_void_p), ("coords_capacity", C.c_uint64),
                ("d_normals", C.c_void_p), ("normals_capacity", C.c_uint64),
                ("d_connections", C.c_void_p), ("connections_capacity", C.c_uint64),
                ("sizes", Sizes), ("status", C.c_int)]


class KvsmlInfo(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("veclen", C.c_uint32), ("grid_uniform", C.c_int32), ("data_format", C.c_int32),
                ("byte_swap", C.c_int32), ("has_min_value", C.c_int32), ("has_max_value", C.c_int32),
                ("min_value", C.c_double), ("max_value", C.c_double), ("volume_min", C.c_double),
                ("volume_max", C.c_double), ("has_object_coord", C.c_int32), ("has_external_coord", C.c_int32),
                ("min_object_coord", C.c_float * 3), ("max_object_coord", C.c_float * 3),
                ("min_external_coord", C.c_float * 3), ("max_external_coord", C.c_float * 3)]


class SliceParams(C.Structure):
    _fields_ = [("coefficients", C.c_float * 4), ("min_coord", C.c_float * 3), ("scale", C.c_float * 3),
                ("tf_min", C.c_float), ("tf_max", C.c_float), ("tf_resolution", C.c_int32),
                ("tf_table", C.c_void_p)]


class TuneChoice(C.Structure):
    _fields_ = [("rows", C.c_int32), ("tasks_per_sm", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("scan_threads", C.c_int32)]


class TuneEntry(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("size_class", C.c_int32), ("choice", TuneChoice),
                ("tuned_ms", C.c_double), ("default_ms", C.c_double)]


class AutotuneConfig(C.Structure):
    _fields_ = [("dtypes", C.POINTER(C.c_int32)), ("ndtypes", C.c_int32), ("max_class", C.c_int32),
                ("isovalues", C.c_int32), ("reps", C.c_int32), ("seed", C.c_uint64)]


SIZE_CLASSES = 5

HOST_ALLOC = C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_int32, C.c_uint64)


class KvsmcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


_lib = None


def load(path=LIB_PATH):
    """Load libkvsmc.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libkvsmc.so is not built ({path}); run kvs_gb300.build.build()")
    lib = C.CDLL(path)
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32
    sig = {
        "kvsmc_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "kvsmc_destroy": (None, [vp]),
        "kvsmc_status_string": (C.c_char_p, [C.c_int]),
        "kvsmc_last_error": (C.c_char_p, [vp]),
        "kvsmc_stream": (vp, [vp]),
        "kvsmc_set_stream": (C.c_int, [vp, vp]),
        "kvsmc_synchronize": (C.c_int, [vp]),
        "kvsmc_kernel_launches": (u64, [vp]),
        "kvsmc_volume_upload": (C.c_int, [vp, vp, C.c_int, u32, u32, u32, C.POINTER(vp)]),
        "kvsmc_volume_from_device": (C.c_int, [vp, vp, C.c_int, u32, u32, u32, C.POINTER(vp)]),
        "kvsmc_volume_update": (C.c_int, [vp, vp, vp]),
        "kvsmc_volume_free": (None, [vp, vp]),
        "kvsmc_volume_minmax": (C.c_int, [vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "kvsmc_count": (C.c_int, [vp, vp, C.POINTER(Params), C.POINTER(Sizes)]),
        "kvsmc_extract_device": (C.c_int, [vp, vp, C.POINTER(Params), vp, u64, vp, u64, vp, u64,
                                           C.POINTER(Sizes)]),
        "kvsmc_marching_cubes_host": (C.c_int, [vp, vp, C.c_int, u32, u32, u32, C.POINTER(Params),
                                                HOST_ALLOC, vp, C.POINTER(Sizes)]),
        "kvsmc_count_batch": (C.c_int, [vp, C.POINTER(Request), i32]),
        "kvsmc_extract_batch": (C.c_int, [vp, C.POINTER(Request), i32]),
        "kvsmc_set_kernel_path": (C.c_int, [vp, i32]),
        "kvsmc_selftest_interpolation": (C.c_int, [vp, u64, u64, C.POINTER(u64), C.POINTER(u64),
                                                   C.POINTER(u64)]),
        "kvsmc_selftest_cells": (C.c_int, [vp, u64, u64, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
        "kvsmc_extract_batch_host": (C.c_int, [vp, vp, C.c_int, u32, u32, u32, C.POINTER(Params), i32,
                                               HOST_ALLOC, vp, C.POINTER(Sizes)]),
        "kvsmc_extract_noalloc": (C.c_int, [vp, C.c_int, u32, u32, u32, C.POINTER(Params), vp, u64, vp, u64,
                                            vp, C.POINTER(Sizes)]),
        "kvsmc_server_create": (C.c_int, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "kvsmc_server_submit": (C.c_int, [vp, vp, C.POINTER(Params), C.POINTER(u64)]),
        "kvsmc_server_poll": (i32, [vp, C.POINTER(Completion), i32, i32]),
        "kvsmc_server_release": (C.c_int, [vp, u64]),
        "kvsmc_server_stats": (C.c_int, [vp, C.POINTER(u64)]),
        "kvsmc_server_destroy": (None, [vp]),
        "kvsmc_copy_to_host": (C.c_int, [vp, vp, vp, u64]),
        "kvsmc_plan_create": (C.c_int, [vp, C.POINTER(Request), i32, C.POINTER(vp)]),
        "kvsmc_plan_launch": (C.c_int, [vp, vp]),
        "kvsmc_plan_wait": (C.c_int, [vp, C.POINTER(Request), i32]),
        "kvsmc_plan_kernels": (u64, [vp]),
        "kvsmc_plan_destroy": (None, [vp]),
        "kvsmc_stl_records": (C.c_int, [vp, i32, vp, vp, vp, u64, u64, vp]),
        "kvsmc_volume_download": (C.c_int, [vp, vp, vp]),
        "kvsmc_slice_count": (C.c_int, [vp, vp, C.POINTER(SliceParams), C.POINTER(u64)]),
        "kvsmc_slice_extract_device": (C.c_int, [vp, vp, C.POINTER(SliceParams), vp, u64, vp, u64, vp, u64,
                                                 C.POINTER(u64)]),
        "kvsmc_slice_plane": (C.c_int, [vp, vp, C.POINTER(SliceParams), HOST_ALLOC, vp, C.POINTER(u64)]),
        "kvsmc_marching_cells_host": (C.c_int, [vp, C.c_int, vp, C.c_int, u64, vp, vp, u64, C.c_double, i32,
                                                C.c_double, C.c_double, HOST_ALLOC, vp, C.POINTER(Sizes)]),
        "kvsmc_marching_cells_device": (C.c_int, [vp, C.c_int, vp, C.c_int, u64, vp, vp, u64, C.c_double, i32,
                                                  C.c_double, C.c_double, vp, u64, vp, u64, C.POINTER(Sizes)]),
        "kvsmc_slice_cells_host": (C.c_int, [vp, C.c_int, vp, C.c_int, u64, vp, vp, u64, C.POINTER(SliceParams),
                                             HOST_ALLOC, vp, C.POINTER(u64)]),
        "kvsmc_cells_bounds": (C.c_int, [vp, C.c_int, vp, u64, vp, u64, vp, vp]),
        "kvsmc_marching_cells_sweep_device": (C.c_int, [vp, C.c_int, vp, C.c_int, u64, vp, vp, u64,
                                                        C.POINTER(C.c_double), i32, i32, C.c_double, C.c_double,
                                                        C.POINTER(vp), C.POINTER(u64), C.POINTER(vp),
                                                        C.POINTER(u64), C.POINTER(Sizes)]),
        "kvsmc_ply_record_bytes": (u32, [i32, i32]),
        "kvsmc_ply_header": (C.c_int64, [u64, i32, i32, C.c_char_p, u64]),
        "kvsmc_ply_records": (C.c_int, [vp, vp, u64, vp, i32, vp, i32, vp]),
        "kvsmc_write_ply": (C.c_int, [vp, C.c_char_p, vp, u64, vp, i32, vp, i32]),
        "kvsmc_write_ply_host": (C.c_int, [vp, C.c_char_p, vp, u64, vp, i32, vp, i32]),
        "kvsmc_kvsml_read_info": (C.c_int, [C.c_char_p, C.POINTER(KvsmlInfo)]),
        "kvsmc_volume_load_kvsml": (C.c_int, [vp, C.c_char_p, C.POINTER(vp), C.POINTER(KvsmlInfo)]),
        "kvsmc_avs_read_info": (C.c_int, [C.c_char_p, C.POINTER(KvsmlInfo)]),
        "kvsmc_volume_load_avs": (C.c_int, [vp, C.c_char_p, C.POINTER(vp), C.POINTER(KvsmlInfo)]),
        "kvsmc_write_stl": (C.c_int, [vp, C.c_char_p, i32, vp, vp, vp, u64, u64]),
        "kvsmc_write_stl_host": (C.c_int, [vp, C.c_char_p, i32, vp, u64, vp, u64, vp, u64]),
        "kvsmc_write_stl_ascii": (C.c_int, [vp, C.c_char_p, i32, vp, vp, vp, u64, u64]),
        "kvsmc_write_stl_ascii_host": (C.c_int, [vp, C.c_char_p, i32, vp, u64, vp, u64, vp, u64]),
        "kvsmc_write_kvsml_polygon": (C.c_int, [vp, C.c_char_p, i32, i32, vp, u64, vp, u64, vp, u64, vp, vp]),
        "kvsmc_size_class": (i32, [u32, u32, u32]),
        "kvsmc_tune_resolve": (C.c_int, [C.POINTER(TuneEntry), i32, C.c_int, u32, u32, u32,
                                         C.POINTER(TuneChoice)]),
        "kvsmc_tuning_set": (C.c_int, [vp, C.POINTER(TuneEntry), i32]),
        "kvsmc_tuning_get": (i32, [vp, C.POINTER(TuneEntry), i32]),
        "kvsmc_tuning_force": (C.c_int, [vp, C.POINTER(TuneChoice)]),
        "kvsmc_autotune": (C.c_int, [vp, C.POINTER(AutotuneConfig), C.POINTER(TuneEntry), i32, C.POINTER(i32)]),
        "kvsmc_profile_enable": (C.c_int, [vp, i32]),
        "kvsmc_profile_read": (i32, [vp, i32, C.POINTER(C.c_char_p), C.POINTER(u64), C.POINTER(C.c_double)]),
        "kvsmc_checksum_words": (C.c_int, [vp, vp, u64, u64, C.POINTER(u64), u64]),
        "kvsmc_set_wait_limit": (C.c_int, [vp, C.c_int64, C.c_int64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def status_string(st):
    return load().kvsmc_status_string(st).decode()


class Context:
    """One libkvsmc context (CUDA stream + scratch arena) on one device."""

    def __init__(self, device=-1):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.kvsmc_create(device, C.byref(h))
        if st != OK:
            raise KvsmcError(st, f"kvsmc_create: {status_string(st)}")
        self.handle = h

    def check(self, st, what):
        if st != OK:
            msg = self.lib.kvsmc_last_error(self.handle).decode()
            raise KvsmcError(st, f"{what}: {status_string(st)}: {msg}")

    @property
    def stream(self):
        return self.lib.kvsmc_stream(self.handle)

    def set_stream(self, cuda_stream_ptr):
        self.check(self.lib.kvsmc_set_stream(self.handle, cuda_stream_ptr), "kvsmc_set_stream")

    def synchronize(self):
        self.check(self.lib.kvsmc_synchronize(self.handle), "kvsmc_synchronize")

    @property
    def kernel_launches(self):
        return int(self.lib.kvsmc_kernel_launches(self.handle))

    def set_kernel_path(self, path):
        self.check(self.lib.kvsmc_set_kernel_path(self.handle, int(path)), "kvsmc_set_kernel_path")

    def profile_enable(self, on=True):
        self.check(self.lib.kvsmc_profile_enable(self.handle, 1 if on else 0), "kvsmc_profile_enable")

    def profile_read(self):
        """{kernel family: (launches, device ms)} since profile_enable()."""
        n = self.lib.kvsmc_profile_read(self.handle, 0, None, None, None)
        names = (C.c_char_p * max(1, n))()
        launches = (C.c_uint64 * max(1, n))()
        ms = (C.c_double * max(1, n))()
        self.lib.kvsmc_profile_read(self.handle, n, names, launches, ms)
        return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(n)}

    def checksum_words(self, ptr, nwords, chunk_words):
        """Per-chunk position-keyed sums of a device array of 32-bit words
        (kvsmc_checksum_words); numpy uint64, one per chunk."""
        nchunks = max(1, (int(nwords) + int(chunk_words) - 1) // int(chunk_words))
        out = np.zeros(nchunks, dtype=np.uint64)
        self.check(self.lib.kvsmc_checksum_words(self.handle, C.c_void_p(int(ptr)), int(nwords), int(chunk_words),
                                                 out.ctypes.data_as(C.POINTER(C.c_uint64)), nchunks),
                   "kvsmc_checksum_words")
        return out

    def set_wait_limit(self, count_polls=-1, emit_polls=-1):
        self.check(self.lib.kvsmc_set_wait_limit(self.handle, int(count_polls), int(emit_polls)),
                   "kvsmc_set_wait_limit")

    def selftest_interpolation(self, n, seed=1):
        t, m, f = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.check(self.lib.kvsmc_selftest_interpolation(self.handle, int(n), int(seed), C.byref(t), C.byref(m),
                                                         C.byref(f)), "kvsmc_selftest_interpolation")
        return t.value, m.value, f.value

    def selftest_cells(self, n, seed=1):
        t, m, f = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.check(self.lib.kvsmc_selftest_cells(self.handle, int(n), int(seed), C.byref(t), C.byref(m),
                                                 C.byref(f)), "kvsmc_selftest_cells")
        return t.value, m.value, f.value

    def close(self):
        if getattr(self, "handle", None):
            self.lib.kvsmc_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceVolume:
    """A volume resident on the device (kvsmc_volume)."""

    def __init__(self, ctx, handle, dtype, shape):
        self.ctx, self.handle, self.dtype, self.shape = ctx, handle, np.dtype(dtype), shape

    @classmethod
    def upload(cls, ctx, values):
        v = np.ascontiguousarray(values)
        nz, ny, nx = v.shape
        h = C.c_void_p()
        ctx.check(ctx.lib.kvsmc_volume_upload(ctx.handle, v.ctypes.data, dtype_code(v.dtype), nx, ny, nz,
                                              C.byref(h)), "kvsmc_volume_upload")
        return cls(ctx, h, v.dtype, v.shape)

    @classmethod
    def from_device(cls, ctx, ptr, dtype, shape):
        nz, ny, nx = shape
        h = C.c_void_p()
        ctx.check(ctx.lib.kvsmc_volume_from_device(ctx.handle, C.c_void_p(ptr), dtype_code(dtype), nx, ny, nz,
                                                   C.byref(h)), "kvsmc_volume_from_device")
        return cls(ctx, h, dtype, tuple(shape))

    def download(self):
        """The values as a host array shaped (nz, ny, nx)."""
        out = np.empty(self.shape, self.dtype)
        self.ctx.check(self.ctx.lib.kvsmc_volume_download(self.ctx.handle, self.handle, out.ctypes.data),
                       "kvsmc_volume_download")
        return out

    def minmax(self):
        mn, mx = C.c_double(), C.c_double()
        self.ctx.check(self.ctx.lib.kvsmc_volume_minmax(self.ctx.handle, self.handle, C.byref(mn), C.byref(mx)),
                       "kvsmc_volume_minmax")
        return mn.value, mx.value

    def free(self):
        if self.handle:
            self.ctx.lib.kvsmc_volume_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.ctx.handle:
                self.free()
        except Exception:
            pass


class Server:
    """The request loop (kvsmc_server_*): submit() from any thread, poll()
    completions, fetch() a result to host memory, release() it to return its
    bytes to the budget."""

    def __init__(self, ctx, budget_bytes=0, max_batch=0, workers=0):
        self.ctx = ctx
        cfg = ServerConfig(budget_bytes, max_batch, workers)
        h = C.c_void_p()
        ctx.check(ctx.lib.kvsmc_server_create(ctx.handle, C.byref(cfg), C.byref(h)), "server_create")
        self.handle = h
        self._buf = (Completion * 256)()

    def submit(self, volume, params):
        t = C.c_uint64()
        self.ctx.check(self.ctx.lib.kvsmc_server_submit(self.handle, volume.handle, C.byref(params), C.byref(t)),
                       "server_submit")
        return t.value

    def poll(self, timeout_ms=0):
        k = self.ctx.lib.kvsmc_server_poll(self.handle, self._buf, len(self._buf), int(timeout_ms))
        return [Completion.from_buffer_copy(self._buf[i]) for i in range(k)]

    def fetch(self, c):
        """(coords, normals) of a completion as host float32 arrays."""
        coords = np.empty(c.sizes.ncoords, np.float32)
        normals = np.empty(c.sizes.nnormals, np.float32)
        for a, ptr in ((coords, c.d_coords), (normals, c.d_normals)):
            if a.size:
                self.ctx.check(self.ctx.lib.kvsmc_copy_to_host(self.ctx.handle, a.ctypes.data, ptr, a.nbytes), "copy")
        return coords, normals

    def release(self, ticket):
        self.ctx.check(self.ctx.lib.kvsmc_server_release(self.handle, ticket), "server_release")

    def stats(self):
        v = (C.c_uint64 * 7)()
        self.ctx.check(self.ctx.lib.kvsmc_server_stats(self.handle, v), "server_stats")
        keys = ("submitted", "completed", "batches", "kernel_launches", "held_bytes", "peak_bytes", "budget_waits")
        return dict(zip(keys, (int(x) for x in v)))

    def close(self):
        if self.handle:
            self.ctx.lib.kvsmc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """A replayable batch (kvsmc_plan_*): created once for a request array,
    then launch() + wait() per extraction."""

    def __init__(self, ctx, reqs):
        self.ctx, self.reqs = ctx, reqs
        h = C.c_void_p()
        ctx.check(ctx.lib.kvsmc_plan_create(ctx.handle, reqs, len(reqs), C.byref(h)), "plan_create")
        self.handle = h

    @property
    def kernels(self):
        return int(self.ctx.lib.kvsmc_plan_kernels(self.handle))

    def launch(self, cuda_stream_ptr=None):
        self.ctx.check(self.ctx.lib.kvsmc_plan_launch(self.handle, cuda_stream_ptr), "plan_launch")

    def wait(self, check=True):
        st = self.ctx.lib.kvsmc_plan_wait(self.handle, self.reqs, len(self.reqs))
        if check:
            self.ctx.check(st, "plan_wait")
        return st

    def close(self):
        if self.handle:
            self.ctx.lib.kvsmc_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_params(isolevel, mode, minmax=None, min_coord=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)):
    p = Params()
    p.isolevel = float(isolevel)
    p.mode = int(mode)
    p.has_minmax = 1 if minmax is not None else 0
    if minmax is not None:
        p.min_value, p.max_value = float(minmax[0]), float(minmax[1])
    for k in range(3):
        p.min_coord[k] = float(min_coord[k])
        p.scale[k] = float(scale[k])
    return p


def sizes_dict(s):
    return dict(ntriangles=s.ntriangles, nvertices=s.nvertices, ncoords=s.ncoords, nnormals=s.nnormals,
                nconnections=s.nconnections, min_value=s.min_value, max_value=s.max_value,
                extracted=bool(s.extracted))


def marching_cubes_host(ctx, values, params):
    """kvsmc_marching_cubes_host on a numpy volume; returns (coords, normals, connections, sizes)."""
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    bufs = {}

    def alloc(user, which, count):
        a = np.empty(count, dtype=np.uint32 if which == 2 else np.float32)
        bufs[which] = a
        return a.ctypes.data

    cb = HOST_ALLOC(alloc)
    s = Sizes()
    ctx.check(ctx.lib.kvsmc_marching_cubes_host(ctx.handle, v.ctypes.data, dtype_code(v.dtype), nx, ny, nz,
                                                C.byref(params), cb, None, C.byref(s)),
              "kvsmc_marching_cubes_host")
    empty_f = np.zeros(0, np.float32)
    return (bufs.get(0, empty_f), bufs.get(1, empty_f), bufs.get(2, np.zeros(0, np.uint32)), sizes_dict(s))


CELL_NODES = (4, 8, 5, 6)   # kvsmc_cell_type: tetrahedra, hexahedra, pyramid, prism


def cells_bounds(ctx, cell_type, coords, connections):
    """kvsmc_cells_bounds: (min float32[3], max float32[3]) of an unstructured volume's nodes."""
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(connections, np.uint32).reshape(-1)
    npc = CELL_NODES[int(cell_type)]
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    ctx.check(ctx.lib.kvsmc_cells_bounds(ctx.handle, int(cell_type), c.ctypes.data, c.size // 3,
                                         k.ctypes.data if k.size else None, k.size // npc, lo.ctypes.data,
                                         hi.ctypes.data), "kvsmc_cells_bounds")
    return lo, hi


def marching_cells_host(ctx, cell_type, values, coords, connections, isolevel, minmax=None):
    """kvsmc_marching_cells_host: (coords, normals, sizes) of one unstructured volume."""
    v = np.ascontiguousarray(values).reshape(-1)
    c = np.ascontiguousarray(coords, np.float32).reshape(-1)
    k = np.ascontiguousarray(connections, np.uint32).reshape(-1)
    npc = CELL_NODES[int(cell_type)]
    if c.size != 3 * v.size or k.size % npc:
        raise ValueError("coords / connections do not match the node count / cell type")
    bufs = {}

    def alloc(user, which, count):
        a = np.empty(count, dtype=np.float32)
        bufs[which] = a
        return a.ctypes.data

    cb = HOST_ALLOC(alloc)
    s = Sizes()
    ctx.check(ctx.lib.kvsmc_marching_cells_host(
        ctx.handle, int(cell_type), v.ctypes.data, dtype_code(v.dtype), v.size, c.ctypes.data,
        k.ctypes.data if k.size else None, k.size // npc, float(isolevel), 1 if minmax is not None else 0,
        float(minmax[0]) if minmax is not None else 0.0, float(minmax[1]) if minmax is not None else 0.0,
        cb, None, C.byref(s)), "kvsmc_marching_cells_host")
    empty_f = np.zeros(0, np.float32)
    return bufs.get(0, empty_f), bufs.get(1, empty_f), sizes_dict(s)


def extract_batch_host(ctx, values, params_list, buffer_for=None):
    """kvsmc_extract_batch_host: one host volume, several requests.

    buffer_for(request, which, count) may return a preallocated numpy array of
    at least `count` elements (e.g. pinned memory) to receive that output;
    otherwise a fresh numpy array is allocated.  Returns one dict per request.
    """
    v = np.ascontiguousarray(values)
    nz, ny, nx = v.shape
    n = len(params_list)
    ps = (Params * max(1, n))(*params_list)
    sizes = (Sizes * max(1, n))()
    bufs = {}

    def alloc(user, which, count):
        req, kind = divmod(which, 3)
        a = buffer_for(req, kind, count) if buffer_for is not None else None
        if a is None:
            a = np.empty(count, dtype=np.uint32 if kind == 2 else np.float32)
        bufs[(req, kind)] = a
        return a.ctypes.data

    cb = HOST_ALLOC(alloc)
    ctx.check(ctx.lib.kvsmc_extract_batch_host(ctx.handle, v.ctypes.data, dtype_code(v.dtype), nx, ny, nz, ps, n, cb,
                                               None, sizes), "kvsmc_extract_batch_host")
    out = []
    for i in range(n):
        s = sizes_dict(sizes[i])
        e = np.zeros(0, np.float32)
        out.append(dict(coords=bufs.get((i, 0), e)[:s["ncoords"]], normals=bufs.get((i, 1), e)[:s["nnormals"]],
                        connections=bufs.get((i, 2), np.zeros(0, np.uint32))[:s["nconnections"]], sizes=s))
    return out
