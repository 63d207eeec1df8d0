"""Bounded device waits that run out.

Every wait of the streaming kernels for a staged node plane is bounded; when it
gives up the kernel records a status word, waits (under its own limit) for its
copies still in flight and stops, and the call returns KVSMC_ERR_TIMEOUT -- the
C-ABI form of the reference's convention of reporting an error and returning a
null result (MarchingCubes.cpp:50-67).  Here kvsmc_set_wait_limit makes those
waits give up at once (a limit of 0 polls: no fault, no hang, the copies still
land), first in the count kernel, then in the emit kernel, and the next normal
extraction on the same context must give the same bits as a fresh context.
"""
import ctypes as C

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _extract(ctx, vol, params):
    s = _abi.Sizes()
    st = ctx.lib.kvsmc_count(ctx.handle, vol.handle, C.byref(params), C.byref(s))
    if st != _abi.OK:
        return st, None, None
    n = max(1, s.ntriangles)
    c = torch.empty(9 * n, dtype=torch.float32, device="cuda")
    nn = torch.empty(3 * n, dtype=torch.float32, device="cuda")
    st = ctx.lib.kvsmc_extract_device(ctx.handle, vol.handle, C.byref(params), c.data_ptr(), 9 * n,
                                      nn.data_ptr(), 3 * n, None, 0, C.byref(s))
    torch.cuda.synchronize()
    if st != _abi.OK:
        return st, None, None
    return st, c[:s.ncoords].cpu().numpy(), nn[:s.nnormals].cpu().numpy()


def _batch(ctx, vol, isos):
    reqs = (_abi.Request * len(isos))()
    for i, iso in enumerate(isos):
        reqs[i].volume = vol.handle
        reqs[i].params = _abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL)
    st = ctx.lib.kvsmc_count_batch(ctx.handle, reqs, len(isos))
    if st != _abi.OK:
        return st, None
    bufs = []
    for i in range(len(isos)):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        n = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        bufs.append((c, n, s.ncoords, s.nnormals))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = n.data_ptr(), s.nnormals
    st = ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, len(isos))
    torch.cuda.synchronize()
    if st != _abi.OK:
        return st, None
    return st, [(c[:a].cpu().numpy(), n[:b].cpu().numpy()) for c, n, a, b in bufs]


@pytest.mark.parametrize("dtype", [np.float32, np.uint8])
def test_wait_timeout_reported_and_context_recovers(dtype):
    v = S.to_numpy(S.fbm((48, 56, 72), seed=13, device="cuda"))
    if np.dtype(dtype) != np.float32:
        v = np.round(v * 255.0).astype(dtype)
    iso = float(v.min()) + 0.47 * (float(v.max()) - float(v.min()))
    isos = [float(v.min()) + f * (float(v.max()) - float(v.min())) for f in (0.3, 0.5, 0.7)]
    params = _abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL)

    fresh = _abi.Context(0)
    fvol = _abi.DeviceVolume.upload(fresh, v)
    st, ref_c, ref_n = _extract(fresh, fvol, params)
    assert st == _abi.OK and ref_c.size > 0
    st, ref_b = _batch(fresh, fvol, isos)
    assert st == _abi.OK

    ctx = _abi.Context(0)
    vol = _abi.DeviceVolume.upload(ctx, v)
    # the count kernel's waits give up
    ctx.set_wait_limit(0, -1)
    st, _, _ = _extract(ctx, vol, params)
    assert st == _abi.ERR_TIMEOUT, _abi.status_string(st)
    st, _ = _batch(ctx, vol, isos)
    assert st == _abi.ERR_TIMEOUT, _abi.status_string(st)
    # the emit kernel's waits give up (the count pass completes)
    ctx.set_wait_limit(-1, 0)
    st, _, _ = _extract(ctx, vol, params)
    assert st == _abi.ERR_TIMEOUT, _abi.status_string(st)
    st, _ = _batch(ctx, vol, isos)
    assert st == _abi.ERR_TIMEOUT, _abi.status_string(st)
    # back to the built-in limit: the same context gives the fresh context's bits
    ctx.set_wait_limit(-1, -1)
    st, c, n = _extract(ctx, vol, params)
    assert st == _abi.OK
    assert same_bits(c, ref_c), first_diff(c, ref_c)
    assert same_bits(n, ref_n), first_diff(n, ref_n)
    st, got = _batch(ctx, vol, isos)
    assert st == _abi.OK
    for (c, n), (rc, rn) in zip(got, ref_b):
        assert same_bits(c, rc), first_diff(c, rc)
        assert same_bits(n, rn), first_diff(n, rn)
    vol.free()
    fvol.free()
    ctx.close()
    fresh.close()


def test_shared_vertex_wait_timeout_and_recovery():
    """The shared-vertex node passes' waits (count, then emit) give up the same way."""
    v = S.to_numpy(S.fbm((40, 48, 64), seed=3, device="cuda"))
    params = _abi.make_params(0.5, _abi.MODE_SHARED_VERTEX_NORMAL)
    fresh = _abi.Context(0)
    fvol = _abi.DeviceVolume.upload(fresh, v)
    ref = _abi.marching_cubes_host(fresh, v, params)
    ctx = _abi.Context(0)
    for limits in ((0, -1), (-1, 0)):
        ctx.set_wait_limit(*limits)
        with pytest.raises(_abi.KvsmcError) as e:
            _abi.marching_cubes_host(ctx, v, params)
        assert e.value.status == _abi.ERR_TIMEOUT
    ctx.set_wait_limit(-1, -1)
    got = _abi.marching_cubes_host(ctx, v, params)
    for a, b in zip(got[:3], ref[:3]):
        assert same_bits(a, b), first_diff(a, b)
    fvol.free()
    ctx.close()
    fresh.close()
