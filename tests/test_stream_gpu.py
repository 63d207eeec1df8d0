"""Streaming kernels (batched, TMA-staged) against the gather kernels and the oracle.

The gather kernels are themselves checked bit-for-bit against the oracle in
test_parity_gpu.py; here every streaming result must equal them bit for bit,
alone and inside batches of mixed volumes, dtypes and isolevels.
"""
import ctypes as C

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def extract_batch(ctx, vols, params_list, path):
    """Run kvsmc_extract_batch with device outputs sized by a count pass."""
    ctx.set_kernel_path(path)
    n = len(params_list)
    reqs = (_abi.Request * n)()
    for i, (v, p) in enumerate(zip(vols, params_list)):
        reqs[i].volume = v.handle
        reqs[i].params = p
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count_batch")
    bufs = []
    for i in range(n):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        k = torch.empty(max(1, s.nconnections), dtype=torch.int32, device="cuda")
        bufs.append((c, nn, k, s.ncoords, s.nnormals, s.nconnections))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
        reqs[i].d_connections, reqs[i].connections_capacity = k.data_ptr(), s.nconnections
    ctx.check(ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, n), "extract_batch")
    ctx.set_kernel_path(_abi.PATH_AUTO)
    out = []
    for i, (c, nn, k, a, b, d) in enumerate(bufs):
        out.append(dict(coords=c[:a].cpu().numpy(), normals=nn[:b].cpu().numpy(),
                        connections=k[:d].cpu().numpy().view(np.uint32), ntri=reqs[i].sizes.ntriangles,
                        status=reqs[i].status))
    return out


def compare(a, b, tag):
    assert a["ntri"] == b["ntri"], (tag, a["ntri"], b["ntri"])
    assert same_bits(a["coords"], b["coords"]), (tag, "coords", first_diff(a["coords"], b["coords"]))
    assert same_bits(a["normals"], b["normals"]), (tag, "normals", first_diff(a["normals"], b["normals"]))


def test_fp32_interpolation_selfcheck(kvsmc_ctx):
    """The FP32 fast path never disagrees with the FP64 sequence."""
    tested, mism, fall = kvsmc_ctx.selftest_interpolation(40_000_000, seed=7)
    assert tested > 10_000_000
    assert mism == 0, (tested, mism, fall)
    assert fall < tested * 0.03, (tested, fall)   # two of the ten distributions are near-degenerate on purpose


def _fields():
    rng = np.random.default_rng(0)
    yield "blobs f32", S.to_numpy(S.gaussian_blobs((45, 60, 70), seed=1)), [0.5, 0.3, 0.7]
    yield "fbm f32", S.to_numpy(S.fbm((40, 50, 300), seed=2)), [0.2 + 0.04 * k for k in range(16)]
    yield "phantom u8", S.to_numpy(S.ellipsoid_phantom((33, 47, 61), np.uint8, seed=3)), [40.5, 100.0, 180.25]
    yield "phantom u16", S.to_numpy(S.ellipsoid_phantom((30, 70, 90), np.uint16, seed=4)), [12000.5, 30000.0]
    yield "noise i8", rng.integers(-100, 100, (20, 21, 22)).astype(np.int8), [0.5, -3.0, 10.25]
    yield "noise i16", rng.integers(-3000, 3000, (17, 19, 520)).astype(np.int16), [0.0, 100.5]
    yield "wide f32", S.to_numpy(S.fbm((6, 9, 1100), seed=5)), [0.5]
    yield "nan f32", _with_nan(S.to_numpy(S.gaussian_blobs((20, 30, 40), seed=6))), [0.4]
    # mostly empty space (one small feature): most bricks are skipped
    yield "sparse f32", _sparse(), [0.5, 0.1]
    # widths that keep one 256-cell row per warp (199 and 449 cells), odd and even row counts
    yield "one-row f32", S.to_numpy(S.gaussian_blobs((21, 33, 200), seed=7)), [0.5, 0.2]
    yield "one-row u8", S.to_numpy(S.ellipsoid_phantom((15, 22, 450), np.uint8, seed=8)), [90.5, 160.0]


def _sparse():
    v = np.zeros((70, 45, 300), np.float32)
    b = S.to_numpy(S.gaussian_blobs((12, 10, 30), seed=9))
    v[40:52, 20:30, 200:230] = b
    return v


def _with_nan(v):
    v = v.copy()
    v[3, 4, 5] = np.nan
    v[10, 2, 30] = np.nan
    return v


@pytest.mark.parametrize("name,v,isos", list(_fields()), ids=[f[0] for f in _fields()])
def test_stream_equals_gather(kvsmc_ctx, name, v, isos):
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    mn, mx = vol.minmax()
    ps = [_abi.make_params(i, 0) for i in isos]
    a = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_AUTO)
    b = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_GATHER)
    for i, iso in enumerate(isos):
        compare(a[i], b[i], f"{name} iso={iso}")
    # preset narrower min/max: clamped interpolation (FP64 fallback on the edges it touches)
    ps = [_abi.make_params(i, 0, minmax=(mn + 0.2 * (mx - mn), mx - 0.2 * (mx - mn))) for i in isos[:2]]
    a = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_AUTO)
    b = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_GATHER)
    for i in range(len(ps)):
        compare(a[i], b[i], f"{name} clamp {i}")


def test_stream_matches_oracle(oracle_lib, kvsmc_ctx):
    v = S.to_numpy(S.fbm((64, 80, 96), seed=9))
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    isos = [0.25, 0.5, 0.61]
    out = extract_batch(kvsmc_ctx, [vol] * 3, [_abi.make_params(i, 0) for i in isos], _abi.PATH_AUTO)
    for i, iso in enumerate(isos):
        o = oracle_lib.extract(v, iso, 0, float(v.min()), float(v.max()))
        assert same_bits(out[i]["coords"], o["coords"]), first_diff(out[i]["coords"], o["coords"])
        assert same_bits(out[i]["normals"], o["normals"]), first_diff(out[i]["normals"], o["normals"])


def test_uneven_batch(kvsmc_ctx):
    """Many volumes of uneven shapes and dtypes in one batch = each alone."""
    rng = np.random.default_rng(12)
    vols, params = [], []
    for i in range(24):
        shape = tuple(int(s) for s in rng.integers(2, 70, 3))
        dt = [np.uint8, np.uint16, np.float32][i % 3]
        v = S.to_numpy(S.ellipsoid_phantom(shape, dt, seed=100 + i))
        dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
        lo, hi = dv.minmax()
        for _ in range(1 + i % 3):
            vols.append(dv)
            params.append(_abi.make_params(lo + rng.uniform(0.2, 0.8) * (hi - lo), 0))
    batch = extract_batch(kvsmc_ctx, vols, params, _abi.PATH_AUTO)
    for i in range(len(params)):
        alone = extract_batch(kvsmc_ctx, [vols[i]], [params[i]], _abi.PATH_GATHER)[0]
        compare(batch[i], alone, f"request {i}")


def test_more_isolevels_than_a_group(kvsmc_ctx):
    v = S.to_numpy(S.fbm((30, 40, 50), seed=13))
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    isos = list(np.linspace(0.1, 0.9, 37))
    a = extract_batch(kvsmc_ctx, [vol] * len(isos), [_abi.make_params(i, 0) for i in isos], _abi.PATH_AUTO)
    b = extract_batch(kvsmc_ctx, [vol] * len(isos), [_abi.make_params(i, 0) for i in isos], _abi.PATH_GATHER)
    for i in range(len(isos)):
        compare(a[i], b[i], f"iso {i}")


def test_capacity_error_reports_sizes(kvsmc_ctx):
    v = S.to_numpy(S.fbm((30, 30, 30), seed=3))
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    p = _abi.make_params(0.5, 0)
    s = _abi.Sizes()
    c = torch.empty(9, dtype=torch.float32, device="cuda")
    st = kvsmc_ctx.lib.kvsmc_extract_device(kvsmc_ctx.handle, vol.handle, C.byref(p), c.data_ptr(), 9,
                                            c.data_ptr(), 3, None, 0, C.byref(s))
    assert st == _abi.ERR_CAPACITY
    assert s.ntriangles > 1 and s.ncoords == 9 * s.ntriangles


def test_clustered_isolevels(kvsmc_ctx):
    """Equal and nearly equal isolevels in one batch (several thresholds in one
    lookup bucket) and node values exactly on thresholds."""
    v = (np.round(S.to_numpy(S.fbm((24, 37, 290), seed=21)) * 64.0) / 64.0).astype(np.float32)
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    isos = [0.5, 0.5, 0.5 + 1e-7, 0.5 + 1e-4, 0.5 + 2e-4, 0.25, 0.25 + 1 / 64, 0.75, 0.75, 31 / 64, 33 / 64]
    ps = [_abi.make_params(i, 0) for i in isos]
    a = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_AUTO)
    b = extract_batch(kvsmc_ctx, [vol] * len(ps), ps, _abi.PATH_GATHER)
    for i, iso in enumerate(isos):
        compare(a[i], b[i], f"f32 iso={iso}")
    u = S.to_numpy(S.ellipsoid_phantom((21, 33, 100), np.uint8, seed=22))
    uvol = _abi.DeviceVolume.upload(kvsmc_ctx, u)
    isos = [100.0, 100.0, 100.5, 101.0, 99.9, 100.25, 20.0, 21.0]
    ps = [_abi.make_params(i, 0) for i in isos]
    a = extract_batch(kvsmc_ctx, [uvol] * len(ps), ps, _abi.PATH_AUTO)
    b = extract_batch(kvsmc_ctx, [uvol] * len(ps), ps, _abi.PATH_GATHER)
    for i, iso in enumerate(isos):
        compare(a[i], b[i], f"u8 iso={iso}")
