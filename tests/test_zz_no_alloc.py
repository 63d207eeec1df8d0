"""kvsmc_extract_noalloc: the extraction for callers that may not allocate
device memory (a plugin whose host application owns the device-memory budget,
or a frame loop where cudaMalloc/cudaFree would synchronize the device).

It is called through the C ABI on a caller-owned device volume and caller-owned
outputs and must give, bit for bit, what kvsmc_extract_device gives, on two
calls in a row (the second reuses the static scratch the first one left).
Collected last on purpose; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _existing_entry_point(ctx, vol, params):
    s = _abi.Sizes()
    ctx.check(ctx.lib.kvsmc_count(ctx.handle, vol.handle, C.byref(params), C.byref(s)), "kvsmc_count")
    c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
    n = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.kvsmc_extract_device(ctx.handle, vol.handle, C.byref(params), c.data_ptr(), s.ncoords,
                                           n.data_ptr(), s.nnormals, None, 0, C.byref(s)), "kvsmc_extract_device")
    torch.cuda.synchronize()
    return c[:s.ncoords].cpu().numpy(), n[:s.nnormals].cpu().numpy(), s.ntriangles


def _field(shape, dtype, seed):
    """fbm in [0, 1] as float32, or spread over an integer type's range."""
    f = S.fbm(shape, seed=seed, device="cuda")
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return S.to_numpy(f)
    info = np.iinfo(dt)
    return S.to_numpy(S._cast(f.double() * (info.max - info.min) + info.min, dt))


def _isos(v, preset):
    lo, hi = float(v.min()), float(v.max())
    return [(lo + 0.45 * (hi - lo), False), (lo + 0.6 * (hi - lo), preset)]


def _check_two_calls(kvsmc_ctx, v):
    lib = _abi.load()
    nz, ny, nx = v.shape
    d_values = torch.from_numpy(v).cuda()
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    stream = torch.cuda.Stream()
    for call, (iso, preset) in enumerate(_isos(v, True)):
        params = _abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL,
                                  minmax=(float(v.min()), float(v.max())) if preset else None)
        ref_c, ref_n, ntri = _existing_entry_point(kvsmc_ctx, vol, params)
        assert ntri > 100
        cap = 9 * ntri + 90
        out_c = torch.full((cap,), -1.0, dtype=torch.float32, device="cuda")
        out_n = torch.full((cap,), -1.0, dtype=torch.float32, device="cuda")
        s = _abi.Sizes()
        st = lib.kvsmc_extract_noalloc(C.c_void_p(d_values.data_ptr()), _abi.dtype_code(v.dtype), nx, ny, nz,
                                       C.byref(params), C.c_void_p(out_c.data_ptr()), cap,
                                       C.c_void_p(out_n.data_ptr()), cap, C.c_void_p(stream.cuda_stream), C.byref(s))
        assert st == _abi.OK, (call, _abi.status_string(st))
        stream.synchronize()
        assert s.ntriangles == ntri and s.ncoords == 9 * ntri and s.nnormals == 3 * ntri
        got_c = out_c[:s.ncoords].cpu().numpy()
        got_n = out_n[:s.nnormals].cpu().numpy()
        assert same_bits(got_c, ref_c), (call, first_diff(got_c, ref_c))
        assert same_bits(got_n, ref_n), (call, first_diff(got_n, ref_n))
        # nothing written past the triangles it reported
        assert np.all(out_c[s.ncoords:].cpu().numpy() == -1.0)
    vol.free()


# every value type the call takes; rows of 64 values are 16-byte multiples for each
@pytest.mark.parametrize("dtype", [np.float32, np.int8, np.uint8, np.int16, np.uint16])
def test_noalloc_matches_extract_device(kvsmc_ctx, dtype):
    _check_two_calls(kvsmc_ctx, _field((40, 52, 64), dtype, seed=21))


def test_noalloc_narrow_rows(kvsmc_ctx):
    # 99 cells per row: two 128-cell rows per warp task (the other tiling)
    _check_two_calls(kvsmc_ctx, _field((30, 41, 100), np.float32, seed=5))


def test_noalloc_near_the_limit(kvsmc_ctx):
    # 512^3: intermediates of about 3.2 MB, just inside the 4 MiB array
    _check_two_calls(kvsmc_ctx, _field((512, 512, 512), np.float32, seed=8))


def test_noalloc_refuses_what_it_cannot_take(kvsmc_ctx):
    lib = _abi.load()
    s = _abi.Sizes()
    p = _abi.make_params(0.5, _abi.MODE_DUP_POLYGON_NORMAL)
    x = torch.zeros(8 * 8 * 8, dtype=torch.float32, device="cuda")
    # shared-vertex mode is not offered
    q = _abi.make_params(0.5, _abi.MODE_SHARED_POLYGON_NORMAL)
    assert lib.kvsmc_extract_noalloc(C.c_void_p(x.data_ptr()), 8, 8, 8, 8, C.byref(q), None, 0, None, 0, None,
                                     C.byref(s)) == _abi.ERR_INVALID_ARGUMENT
    # rows that are not 16-byte multiples
    assert lib.kvsmc_extract_noalloc(C.c_void_p(x.data_ptr()), 8, 5, 8, 8, C.byref(p), None, 0, None, 0, None,
                                     C.byref(s)) == _abi.ERR_INVALID_ARGUMENT
    # intermediates beyond the static array: 64 x 2 x 400001 float32 needs one
    # count and one offset for each of 400000 tiles (> 4 MiB).  The array is
    # really that large, so the call stays in bounds whatever it does.
    nz = 400_001
    tall = torch.zeros(64 * 2 * nz, dtype=torch.float32, device="cuda")
    assert lib.kvsmc_extract_noalloc(C.c_void_p(tall.data_ptr()), 8, 64, 2, nz, C.byref(p), None, 0, None, 0,
                                     None, C.byref(s)) == _abi.ERR_TOO_LARGE
