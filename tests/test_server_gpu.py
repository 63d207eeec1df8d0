"""The request loop (kvsmc_server_*): continuous batching over resident volumes.

Each result must be the same bits whether the request ran alone (one plain
kvsmc_extract_device call) or inside whatever batch the server formed while
other requests were arriving; the output budget must hold back batches
until results are released, and refuse a result that can never fit.
"""
import threading
import time

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _volumes(ctx):
    vs = [S.to_numpy(S.fbm((40, 52, 64), seed=41)),
          S.to_numpy(S.ellipsoid_phantom((33, 47, 150), np.uint16, seed=42)),
          S.to_numpy(S.gaussian_blobs((28, 60, 300), seed=43)),
          S.to_numpy(S.ellipsoid_phantom((50, 31, 90), np.uint8, seed=44))]
    return [_abi.DeviceVolume.upload(ctx, v) for v in vs]


def _alone(ctx, vol, params):
    s = _abi.Sizes()
    ctx.check(ctx.lib.kvsmc_count(ctx.handle, vol.handle, params, s), "count")
    c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
    n = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.kvsmc_extract_device(ctx.handle, vol.handle, params, c.data_ptr(), s.ncoords, n.data_ptr(),
                                           s.nnormals, None, 0, s), "extract_device")
    ctx.synchronize()
    return s.ntriangles, c[:s.ncoords].cpu().numpy(), n[:s.nnormals].cpu().numpy()


def _collect(srv, count, release=True, timeout_s=60.0):
    got = {}
    t_end = time.time() + timeout_s
    while len(got) < count and time.time() < t_end:
        for c in srv.poll(timeout_ms=200):
            got[c.ticket] = (c, srv.fetch(c) if c.status == 0 else None)
            if release:
                srv.release(c.ticket)
    return got


def test_server_mix_equals_alone(kvsmc_ctx):
    vols = _volumes(kvsmc_ctx)
    rng = np.random.default_rng(45)
    reqs = []
    for i in range(64):
        v = vols[int(rng.integers(0, len(vols)))]
        lo, hi = v.minmax()
        reqs.append((v, _abi.make_params(lo + rng.uniform(0.1, 0.9) * (hi - lo), 0)))
    srv = _abi.Server(kvsmc_ctx, budget_bytes=1 << 30, max_batch=16, workers=3)
    tickets = [None] * len(reqs)

    def submit(part):
        for i in part:
            tickets[i] = srv.submit(*reqs[i])

    threads = [threading.Thread(target=submit, args=(range(k, len(reqs), 2),)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got = _collect(srv, len(reqs))
    stats = srv.stats()
    srv.close()
    assert len(got) == len(reqs), stats
    for i, (v, p) in enumerate(reqs):
        c, out = got[tickets[i]]
        assert c.status == 0, (i, c.status)
        ntri, coords, normals = _alone(kvsmc_ctx, v, p)
        assert c.sizes.ntriangles == ntri, (i, c.sizes.ntriangles, ntri)
        assert same_bits(out[0], coords), (i, first_diff(out[0], coords))
        assert same_bits(out[1], normals), (i, first_diff(out[1], normals))
        assert c.submit_s <= c.start_s <= c.done_s
    assert stats["completed"] == len(reqs) and stats["held_bytes"] == 0


def test_server_budget_holds_back_and_refuses(kvsmc_ctx):
    vols = _volumes(kvsmc_ctx)
    v = vols[2]
    lo, hi = v.minmax()
    isos = [lo + f * (hi - lo) for f in (0.3, 0.4, 0.5, 0.6)]
    sizes = []
    for iso in isos:
        s = _abi.Sizes()
        kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_count(kvsmc_ctx.handle, v.handle, _abi.make_params(iso, 0), s), "count")
        sizes.append(48 * s.ntriangles)
    assert min(sizes) > 0
    budget = max(sizes) + min(sizes) // 2    # about one result at a time
    srv = _abi.Server(kvsmc_ctx, budget_bytes=budget, max_batch=2, workers=2)
    tickets = [srv.submit(v, _abi.make_params(iso, 0)) for iso in isos * 2]
    got = _collect(srv, len(tickets))
    stats = srv.stats()
    assert len(got) == len(tickets) and all(got[t][0].status == 0 for t in tickets)
    assert stats["peak_bytes"] <= budget
    srv.close()
    # a result larger than the whole budget can never be admitted
    small = _abi.Server(kvsmc_ctx, budget_bytes=min(sizes) // 2, max_batch=4, workers=1)
    t = small.submit(v, _abi.make_params(isos[2], 0))
    out = _collect(small, 1)
    assert out[t][0].status == _abi.ERR_BUDGET
    small.close()


def test_server_refuses_unserved_requests(kvsmc_ctx):
    vols = _volumes(kvsmc_ctx)
    srv = _abi.Server(kvsmc_ctx)
    with pytest.raises(_abi.KvsmcError):
        srv.submit(vols[0], _abi.make_params(0.5, _abi.MODE_SHARED_POLYGON_NORMAL))
    srv.close()
