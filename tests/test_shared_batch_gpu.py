"""Batches of shared-vertex requests: one streaming triangle count for all of them.

kvsmc_extract_batch / kvsmc_count_batch / kvsmc_extract_batch_host count the
triangles and vertices of every shared-vertex request of a batch (PolygonNormal
without duplication, VertexNormal) in one streaming pass per volume group (up
to 16 isolevels share one read of the volume), write the group's vertices and
rank words in one node emit pass, and each request's connection pass takes its
isolevel's offsets from that count.  The results must be the
oracle's (oracle/mc_oracle.c) bit for bit, and equal each request run alone
(which counts on its own), including volumes that do not take the shared
count (two rows per task), more than 16 isolevels on one volume, mixed modes
and value types, and a count whose bounded waits give up.
"""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits
from .test_stream_gpu import extract_batch

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _same(a, b, tag):
    assert a["ntri"] == b["ntri"], (tag, a["ntri"], b["ntri"])
    for k in ("coords", "normals"):
        assert same_bits(a[k], b[k]), (tag, k, first_diff(a[k], b[k]))
    assert np.array_equal(a["connections"], b["connections"]), tag


def test_shared_batch_matches_the_oracle(kvsmc_ctx, oracle_lib):
    v = S.to_numpy(S.fbm((40, 48, 200), seed=21, device="cuda"))   # 199 cells per row: one row per task
    lo, hi = float(v.min()), float(v.max())
    reqs = [(0.35, 1), (0.4, 2), (0.45, 0), (0.5, 2), (0.55, 1), (0.62, 2)]
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    out = extract_batch(kvsmc_ctx, [vol] * len(reqs), [_abi.make_params(x, m) for x, m in reqs], _abi.PATH_AUTO)
    for (x, m), o in zip(reqs, out):
        assert o["status"] == _abi.OK
        ref = oracle_lib.extract(v, x, m, lo, hi)
        assert same_bits(o["coords"], ref["coords"]), (x, m, first_diff(o["coords"], ref["coords"]))
        assert same_bits(o["normals"], ref["normals"]), (x, m, first_diff(o["normals"], ref["normals"]))
        assert np.array_equal(o["connections"], ref["connections"].view(np.uint32)), (x, m)
    vol.free()


def test_shared_batch_equals_alone(kvsmc_ctx):
    """Groups of more than 16 isolevels, four value types, a two-rows-per-task
    volume, rows of several segments, and a row whose last node starts a
    segment of its own (its requests count their vertices on their own)."""
    rng = np.random.default_rng(5)
    vols, params = [], []
    f = S.fbm((40, 44, 256), seed=8, device="cuda")
    cases = [
        (S.to_numpy(f), 20),                                                          # f32, 2 groups
        (S.to_numpy(S._cast(f.double() * 255.0, np.uint8)), 3),                       # u8
        (S.to_numpy(S._cast(f.double() * 65535.0, np.uint16)), 3),                    # u16
        (S.to_numpy(S._cast(f.double() * 60000.0 - 30000.0, np.int16)), 2),           # i16
        (S.to_numpy(S.fbm((36, 40, 100), seed=9, device="cuda")), 3),                 # 99 cells: 2 rows per task
        (S.to_numpy(S.fbm((20, 24, 700), seed=10, device="cuda")), 3),                # 3 segments, the last partial
        (S.to_numpy(S.fbm((18, 22, 257), seed=11, device="cuda")), 2),                # node 256 alone in a segment
    ]
    for v, n in cases:
        dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
        lo, hi = dv.minmax()
        for _ in range(n):
            vols.append(dv)
            params.append(_abi.make_params(lo + rng.uniform(0.25, 0.75) * (hi - lo), int(rng.integers(1, 3))))
    batch = extract_batch(kvsmc_ctx, vols, params, _abi.PATH_AUTO)
    for i in range(len(params)):
        assert batch[i]["status"] == _abi.OK
        alone = extract_batch(kvsmc_ctx, [vols[i]], [params[i]], _abi.PATH_AUTO)[0]
        _same(batch[i], alone, f"request {i}")
    for dv in {id(d): d for d in vols}.values():
        dv.free()


def test_shared_batch_count_timeout_and_recovery():
    """The shared count's plane waits, then the grouped node emit's, give up
    with KVSMC_ERR_TIMEOUT for every request they cover; the next batch on the
    same context is exact again."""
    v = S.to_numpy(S.fbm((30, 40, 150), seed=3, device="cuda"))
    ctx = _abi.Context(0)
    vol = _abi.DeviceVolume.upload(ctx, v)
    params = [_abi.make_params(x, _abi.MODE_SHARED_VERTEX_NORMAL) for x in (0.4, 0.5, 0.6)]
    ref = [extract_batch(ctx, [vol], [p], _abi.PATH_AUTO)[0] for p in params]
    for limits in ((0, -1), (-1, 0)):
        ctx.set_wait_limit(*limits)
        with pytest.raises(_abi.KvsmcError) as e:
            extract_batch(ctx, [vol] * 3, params, _abi.PATH_AUTO)
        assert e.value.status == _abi.ERR_TIMEOUT
    ctx.set_wait_limit(-1, -1)
    got = extract_batch(ctx, [vol] * 3, params, _abi.PATH_AUTO)
    for a, b in zip(got, ref):
        _same(a, b, "after timeout")
    vol.free()
    ctx.close()


def test_host_batch_shared_requests_match_alone(kvsmc_ctx):
    v = S.to_numpy(S.gaussian_blobs((40, 50, 160), seed=12, device="cuda"))
    params = [_abi.make_params(x, m) for x, m in ((0.3, 2), (0.45, 1), (0.5, 0), (0.6, 2))]
    out = _abi.extract_batch_host(kvsmc_ctx, v, params)
    for k, p in enumerate(params):
        alone = _abi.extract_batch_host(kvsmc_ctx, v, [p])[0]
        for key in ("coords", "normals"):
            assert same_bits(out[k][key], alone[key]), (k, key, first_diff(out[k][key], alone[key]))
        assert np.array_equal(out[k]["connections"], alone["connections"]), k


def test_shared_batch_capacity_error_leaves_the_others_exact(kvsmc_ctx):
    """A request whose buffers are too small fails alone with KVSMC_ERR_CAPACITY;
    the grouped passes still write the other requests exactly."""
    v = S.to_numpy(S.fbm((30, 36, 180), seed=14, device="cuda"))
    vol = _abi.DeviceVolume.upload(kvsmc_ctx, v)
    params = [_abi.make_params(x, _abi.MODE_SHARED_VERTEX_NORMAL) for x in (0.35, 0.5, 0.65)]
    alone = [extract_batch(kvsmc_ctx, [vol], [p], _abi.PATH_AUTO)[0] for p in params]
    n = len(params)
    reqs = (_abi.Request * n)()
    for i, p in enumerate(params):
        reqs[i].volume = vol.handle
        reqs[i].params = p
    kvsmc_ctx.check(kvsmc_ctx.lib.kvsmc_count_batch(kvsmc_ctx.handle, reqs, n), "count_batch")
    bufs = []
    for i in range(n):
        s = reqs[i].sizes
        short = 3 if i == 1 else 0   # request 1: three coordinates too few
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        k = torch.empty(max(1, s.nconnections), dtype=torch.int32, device="cuda")
        bufs.append((c, nn, k, s.ncoords, s.nnormals, s.nconnections))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords - short
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
        reqs[i].d_connections, reqs[i].connections_capacity = k.data_ptr(), s.nconnections
    st = kvsmc_ctx.lib.kvsmc_extract_batch(kvsmc_ctx.handle, reqs, n)
    assert st == _abi.ERR_CAPACITY
    assert reqs[1].status == _abi.ERR_CAPACITY
    for i in (0, 2):
        assert reqs[i].status == _abi.OK
        c, nn, k, a, b, d = bufs[i]
        got = dict(coords=c[:a].cpu().numpy(), normals=nn[:b].cpu().numpy(),
                   connections=k[:d].cpu().numpy().view(np.uint32), ntri=reqs[i].sizes.ntriangles)
        _same(got, alone[i], f"request {i}")
    vol.free()


@pytest.mark.parametrize("seed", [101, 202, 303])
def test_shared_batch_random_shapes_equal_alone(kvsmc_ctx, seed):
    """Random shapes (rows of one to three segments, the last one partial, or a
    last node alone in a segment; two-row volumes; as few as two planes or rows),
    value types and isolevel sets: every grouped request equals the same request
    run alone."""
    rng = np.random.default_rng(seed)
    vols, params = [], []
    for _ in range(4):
        nx = int(rng.choice([129, 200, 255, 256, 300, 511, 512, 513, 700]))
        ny = int(rng.integers(2, 24))
        nz = int(rng.integers(2, 20))
        dt = [np.uint8, np.uint16, np.int16, np.float32][int(rng.integers(0, 4))]
        f = S.fbm((nz, ny, nx), seed=int(rng.integers(0, 1 << 16)), device="cuda")
        if np.dtype(dt).kind == "f":
            v = S.to_numpy(f)
        else:
            lo, hi = (-30000.0, 30000.0) if np.dtype(dt) == np.int16 else (0.0, 250.0 if dt == np.uint8 else 60000.0)
            v = S.to_numpy(S._cast(f.double() * (hi - lo) + lo, dt))
        dv = _abi.DeviceVolume.upload(kvsmc_ctx, v)
        mn, mx = dv.minmax()
        for _ in range(int(rng.integers(2, 6))):
            vols.append(dv)
            params.append(_abi.make_params(mn + rng.uniform(0.1, 0.9) * (mx - mn), int(rng.integers(1, 3))))
    batch = extract_batch(kvsmc_ctx, vols, params, _abi.PATH_AUTO)
    for i in range(len(params)):
        assert batch[i]["status"] == _abi.OK
        alone = extract_batch(kvsmc_ctx, [vols[i]], [params[i]], _abi.PATH_AUTO)[0]
        _same(batch[i], alone, f"seed {seed} request {i}")
    for dv in {id(d): d for d in vols}.values():
        dv.free()
