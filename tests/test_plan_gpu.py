"""Replayable batch plans (kvsmc_plan_*): one CUDA graph per batch.

Every replay must give exactly what kvsmc_extract_batch gives for the same
requests (which is itself pinned to the gather kernels and the oracle), the
device-side capacity guard must never write past a request's buffers, and a
volume updated in place must be re-read by the next replay.
"""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits
from .test_stream_gpu import compare, extract_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _requests(vols, params, caps=None, slack=0, tri_caps=None):
    """Request array with device outputs sized by a count pass (times `caps`
    when given, or `tri_caps` triangles), plus `slack` sentinel floats past
    each capacity."""
    ctx = vols[0].ctx
    n = len(params)
    reqs = (_abi.Request * n)()
    for i, (v, p) in enumerate(zip(vols, params)):
        reqs[i].volume = v.handle
        reqs[i].params = p
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count_batch")
    bufs = []
    for i in range(n):
        t = reqs[i].sizes.ntriangles
        cap = tri_caps[i] if tri_caps is not None else (t if caps is None else int(t * caps[i]))
        c = torch.full((max(1, 9 * cap + slack),), -7.0, dtype=torch.float32, device="cuda")
        nn = torch.full((max(1, 3 * cap + slack),), -7.0, dtype=torch.float32, device="cuda")
        bufs.append((c, nn, cap))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), 9 * cap
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), 3 * cap
    return reqs, bufs


def _mixed(ctx, seed):
    rng = np.random.default_rng(seed)
    vols, params, hosts = [], [], []
    for i in range(14):
        shape = tuple(int(s) for s in rng.integers(3, 60, 3))
        dt = [np.uint8, np.uint16, np.float32, np.int8, np.int16][i % 5]
        if dt in (np.int8, np.int16):
            v = rng.integers(-100, 100, shape).astype(dt)
        else:
            v = S.to_numpy(S.ellipsoid_phantom(shape, dt, seed=seed + i))
        dv = _abi.DeviceVolume.upload(ctx, v)
        lo, hi = dv.minmax()
        for _ in range(1 + i % 3):
            vols.append(dv)
            hosts.append(v)
            params.append(_abi.make_params(lo + rng.uniform(0.2, 0.8) * (hi - lo), 0))
    return vols, params, hosts


def test_plan_replay_equals_batch(kvsmc_ctx):
    vols, params, _ = _mixed(kvsmc_ctx, 30)
    ref = extract_batch(kvsmc_ctx, vols, params, _abi.PATH_AUTO)
    reqs, bufs = _requests(vols, params)
    plan = _abi.Plan(kvsmc_ctx, reqs)
    assert plan.kernels >= 6
    for rep in range(3):
        for c, nn, _ in bufs:
            c.fill_(0.0)
            nn.fill_(0.0)
        plan.launch()
        plan.wait()
        for i in range(len(params)):
            assert reqs[i].status == 0
            got = dict(coords=bufs[i][0][:9 * reqs[i].sizes.ntriangles].cpu().numpy(),
                       normals=bufs[i][1][:3 * reqs[i].sizes.ntriangles].cpu().numpy(),
                       ntri=reqs[i].sizes.ntriangles)
            compare(got, ref[i], f"replay {rep} request {i}")
    plan.close()


def test_plan_capacity_guard(kvsmc_ctx):
    """A request whose buffers hold only part of its result gets
    KVSMC_ERR_CAPACITY with the full sizes; nothing past its capacity is
    written; the other requests are unaffected."""
    v = S.to_numpy(S.fbm((30, 41, 77), seed=31))
    dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    isos = [0.3, 0.5, 0.7]
    params = [_abi.make_params(i, 0) for i in isos]
    ref = extract_batch(kvsmc_ctx, [dv] * 3, params, _abi.PATH_AUTO)
    reqs, bufs = _requests([dv] * 3, params, caps=[1.0, 0.5, 1.0], slack=64)
    plan = _abi.Plan(kvsmc_ctx, reqs)
    plan.launch()
    st = plan.wait(check=False)
    assert st == _abi.ERR_CAPACITY
    assert reqs[0].status == 0 and reqs[2].status == 0
    assert reqs[1].status == _abi.ERR_CAPACITY
    assert reqs[1].sizes.ntriangles == ref[1]["ntri"]
    c, nn, cap = bufs[1]
    hc, hn = c.cpu().numpy(), nn.cpu().numpy()
    assert np.all(hc[9 * cap:] == -7.0) and np.all(hn[3 * cap:] == -7.0)
    assert same_bits(hc[:9 * cap], ref[1]["coords"][:9 * cap]), first_diff(hc[:9 * cap], ref[1]["coords"][:9 * cap])
    for i in (0, 2):
        got = dict(coords=bufs[i][0][:9 * reqs[i].sizes.ntriangles].cpu().numpy(),
                   normals=bufs[i][1][:3 * reqs[i].sizes.ntriangles].cpu().numpy(), ntri=reqs[i].sizes.ntriangles)
        compare(got, ref[i], f"request {i}")
    plan.close()


def test_plan_rereads_updated_volume(kvsmc_ctx):
    a = S.to_numpy(S.gaussian_blobs((26, 33, 40), seed=32))
    b = S.to_numpy(S.gaussian_blobs((26, 33, 40), seed=33))
    dv = _abi.DeviceVolume.upload(kvsmc_ctx, a)
    # preset min/max so the plan's frozen range is right for both contents
    lo, hi = float(min(a.min(), b.min())), float(max(a.max(), b.max()))
    params = [_abi.make_params(0.5, 0, minmax=(lo, hi)), _abi.make_params(0.25, 0, minmax=(lo, hi))]
    need = [0, 0]
    for src in (b, a):
        kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_volume_update(kvsmc_ctx.handle, dv.handle, src.ctypes.data), "update")
        r = extract_batch(kvsmc_ctx, [dv, dv], params, _abi.PATH_AUTO)
        need = [max(need[i], r[i]["ntri"]) for i in range(2)]
    reqs, bufs = _requests([dv, dv], params, tri_caps=need)
    plan = _abi.Plan(kvsmc_ctx, reqs)
    for src in (a, b, a):
        kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_volume_update(kvsmc_ctx.handle, dv.handle, src.ctypes.data), "update")
        ref = extract_batch(kvsmc_ctx, [dv, dv], params, _abi.PATH_AUTO)
        plan.launch()
        plan.wait()
        for i in range(2):
            got = dict(coords=bufs[i][0][:9 * reqs[i].sizes.ntriangles].cpu().numpy(),
                       normals=bufs[i][1][:3 * reqs[i].sizes.ntriangles].cpu().numpy(),
                       ntri=reqs[i].sizes.ntriangles)
            compare(got, ref[i], f"request {i}")
    plan.close()


def test_plan_constant_volume_and_rejects(kvsmc_ctx):
    flat = np.full((5, 6, 7), 3.0, np.float32)
    dflat = _abi.DeviceVolume.upload(kvsmc_ctx, flat)
    reqs, _ = _requests([dflat], [_abi.make_params(3.0, 0)])
    plan = _abi.Plan(kvsmc_ctx, reqs)
    assert plan.kernels == 0
    plan.launch()
    plan.wait()
    assert reqs[0].status == 0 and reqs[0].sizes.extracted == 0 and reqs[0].sizes.ntriangles == 0
    plan.close()
    v = S.to_numpy(S.gaussian_blobs((10, 11, 12), seed=34))
    dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    reqs = (_abi.Request * 1)()
    reqs[0].volume = dv.handle
    reqs[0].params = _abi.make_params(0.5, _abi.MODE_SHARED_POLYGON_NORMAL)
    with pytest.raises(_abi.KvsmcError):
        _abi.Plan(kvsmc_ctx, reqs)
