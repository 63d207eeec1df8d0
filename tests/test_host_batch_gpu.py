"""kvsmc_extract_batch_host: one host volume, many requests, host outputs.

The end-to-end call the bench's e2e leg times.  Its streaming requests are
emitted in launches over ranges of cell planes and each range's triangles are
copied to the host on a second stream while the next range is written; the
result must be the oracle's (oracle/mc_oracle.c) bit for bit whatever the split:
one volume with up to 16 isolevels (split), more than 16 (two groups, one
launch), shared-vertex requests in the same call (the gather kernels), and
preallocated (pinned) host buffers like the bench's.
"""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import synthetic as S

from .helpers import first_diff, same_bits

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _oracle(oracle_lib, v, iso, mode, lo, hi):
    o = oracle_lib.extract(v, iso, mode, lo, hi)
    return o


def _check(out, ref, tag):
    assert out["sizes"]["ncoords"] == ref["coords"].size, tag
    assert same_bits(out["coords"], ref["coords"]), (tag, first_diff(out["coords"], ref["coords"]))
    assert same_bits(out["normals"], ref["normals"]), (tag, first_diff(out["normals"], ref["normals"]))
    assert np.array_equal(out["connections"], ref["connections"]), tag


@pytest.mark.parametrize("shape,dtype,niso", [((70, 64, 80), np.float32, 5), ((130, 40, 33), np.uint16, 16),
                                              ((40, 48, 56), np.float32, 20)])
def test_host_batch_matches_the_oracle(kvsmc_ctx, oracle_lib, shape, dtype, niso):
    f = S.fbm(shape, seed=4, device="cuda")
    if np.dtype(dtype) == np.uint16:
        v = S.to_numpy(S._cast(f.double() * 65535.0, np.uint16))
    else:
        v = S.to_numpy(f)
    lo, hi = float(v.min()), float(v.max())
    isos = [lo + (hi - lo) * (0.15 + 0.7 * k / max(1, niso - 1)) for k in range(niso)]
    params = [_abi.make_params(x, _abi.MODE_DUP_POLYGON_NORMAL) for x in isos]
    out = _abi.extract_batch_host(kvsmc_ctx, v, params)
    for k, x in enumerate(isos):
        _check(out[k], _oracle(oracle_lib, v, x, 0, lo, hi), (shape, k))


def test_host_batch_mixed_modes_and_pinned_buffers(kvsmc_ctx, oracle_lib):
    v = S.to_numpy(S.gaussian_blobs((60, 72, 64), seed=9, device="cuda"))
    lo, hi = float(v.min()), float(v.max())
    reqs = [(0.3, 0), (0.5, 1), (0.45, 0), (0.6, 2), (0.7, 0)]
    params = [_abi.make_params(x, m) for x, m in reqs]
    pinned = {}

    def buf(req, kind, count):
        a = torch.empty(count, dtype=torch.int32 if kind == 2 else torch.float32, pin_memory=True).numpy()
        if kind == 2:
            a = a.view(np.uint32)
        pinned[(req, kind)] = a
        return a

    for _ in range(2):   # the second call reuses the context's arenas and copy stream
        out = _abi.extract_batch_host(kvsmc_ctx, v, params, buf)
        for k, (x, m) in enumerate(reqs):
            _check(out[k], _oracle(oracle_lib, v, x, m, lo, hi), (x, m))
