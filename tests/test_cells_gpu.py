"""The unstructured marching mappers on the GPU (kvsmc_marching_cells_host
through kvs_gb300.marching_cells and kvs_gb300.isosurface) against the
fixtures made from the reference MarchingTetrahedra / Hexahedra / Pyramid /
Prism, bit for bit (coordinates, normals, colour, types, the volume's min/max
cache, bounding box), and against the numpy restatement on grids of a
million and more cells."""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import marching_cells as mcells
from kvs_gb300.isosurface import Isosurface
from kvs_gb300.marching_cubes import PolygonObject, TransferFunction
from oracle import cells as ocells

from . import cell_meshes as cm
from .helpers import first_diff, same_bits
from .test_cells_cpu import case_inputs, cells_fixtures

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _volume(ct, v, xyz, conn):
    return mcells.UnstructuredVolumeObject(mcells.MAPPERS_BY_ABI[ct].CELL, v.size, conn.shape[0], 1, xyz, conn, v)


def _run(e, arr, ctx):
    v, xyz, conn = case_inputs(arr, e)
    vol = _volume(e["cell_type"], v, xyz, conn)
    if e["minmax"] is not None:
        vol.setMinMaxValues(*e["minmax"])
    tf = TransferFunction(256)
    if e["tf_range"]:
        tf.setRange(*e["tf_range"])
    nt = PolygonObject.PolygonNormal if e["normal_type"] == "polygon" else PolygonObject.VertexNormal
    if e["form"] == 1:
        m = Isosurface(vol, e["iso"], nt, e["duplication"], tf, context=ctx)
    else:
        m = mcells.MAPPERS_BY_ABI[e["cell_type"]](vol, e["iso"], nt, e["duplication"], tf, context=ctx)
    return m, vol


def test_mappers_match_reference_fixtures(kvsmc_ctx):
    man, arr = cells_fixtures()
    for e in man:
        k = e["key"]
        m, vol = _run(e, arr, kvsmc_ctx)
        assert m.isSuccess() == e["success"], k
        for f, got in (("coords", m.coords()), ("normals", m.normals())):
            want = arr[f"{k}__{f}"]
            assert same_bits(got, want), (k, f, first_diff(got, want))
        assert np.array_equal(m.colors(), arr[f"{k}__colors"]), k
        assert np.array_equal(m.opacities(), arr[f"{k}__opacities"]), k
        assert m.connections().size == 0, k
        assert (m.polygonType(), m.colorType(), m.normalType()) == (
            e["polygon_type"], e["color_type"], e["normal_type_out"]), k
        assert vol.hasMinMaxValues() == e["vol_has_minmax"], k
        assert same_bits(np.array([vol.minValue(), vol.maxValue()]), arr[f"{k}__vol_minmax"]), k
        assert np.array_equal(m.minObjectCoord(), np.float32(e["min_obj"])), k
        assert np.array_equal(m.maxObjectCoord(), np.float32(e["max_obj"])), k
        assert np.array_equal(m.maxExternalCoord(), np.float32(e["max_ext"])), k


@pytest.mark.parametrize("ct", [0, 1, 2, 3])
def test_large_grids_match_oracle(kvsmc_ctx, ct):
    """About 1.5 M tetrahedra, 250 k hexahedra, 1.5 M pyramids, 500 k prisms."""
    xyz, conn = cm.grid(ct, 64, 64, 64, jitter=0.3, seed=40 + ct)
    v = cm.sphere_values(xyz, (30.3, 31.7, 29.1))
    for iso in (12.5, 27.0):
        got_c, got_n, sizes = _abi.marching_cells_host(kvsmc_ctx, ct, v, xyz, conn, iso)
        o = ocells.marching_cells(ct, v, xyz, conn, iso)
        assert sizes["ntriangles"] * 9 == o["coords"].size > 0
        assert (sizes["min_value"], sizes["max_value"]) == (o["vmin"], o["vmax"])
        assert same_bits(got_c, o["coords"]), (ct, iso, first_diff(got_c, o["coords"]))
        assert same_bits(got_n, o["normals"]), (ct, iso, first_diff(got_n, o["normals"]))


def test_all_value_types_on_random_meshes(kvsmc_ctx):
    """Random connectivity (every table case) at a size the fixtures do not
    reach, all ten value types, with and without a preset min/max."""
    rng = np.random.default_rng(5)
    for ct in range(4):
        xyz, conn = cm.random_mesh(ct, 5000, 200000, seed=ct)
        for dt in _abi.DTYPES:
            info = np.iinfo(dt) if np.dtype(dt).kind in "iu" else None
            if info is None:
                v = rng.standard_normal(5000).astype(dt)
                iso = 0.25
            else:
                lo, hi = max(info.min, -1000), min(info.max, 1000)
                v = rng.integers(lo, hi, 5000).astype(dt)
                iso = (lo + hi) / 2 + 0.5
            for mm in (None, (float(v.min()) / 2, float(v.max()) / 2)):
                got_c, got_n, sizes = _abi.marching_cells_host(kvsmc_ctx, ct, v, xyz, conn, iso, mm)
                o = ocells.marching_cells(ct, v, xyz, conn, iso, mm)
                assert same_bits(got_c, o["coords"]), (ct, dt, mm, first_diff(got_c, o["coords"]))
                assert same_bits(got_n, o["normals"]), (ct, dt, mm)


def test_isosurface_default_isolevel_on_unstructured(kvsmc_ctx):
    """Isosurface(volume, normal_type): the isolevel is (max + min) / 2 from the
    device min/max over the cells' nodes."""
    xyz, conn = cm.grid(0, 20, 18, 16, seed=3)
    v = cm.sphere_values(xyz, (9.1, 8.3, 7.7))
    v[0] = 100.0           # node 0 is always in the scan
    vol = _volume(0, v, xyz, conn)
    iso = Isosurface(vol, normal_type=PolygonObject.PolygonNormal, context=kvsmc_ctx)
    lo, hi = ocells.minmax(v, conn, 0)
    assert (vol.minValue(), vol.maxValue()) == (lo, hi) and hi == 100.0
    o = ocells.marching_cells(0, v, xyz, conn, (hi + lo) * 0.5)
    assert o["coords"].size > 0 and same_bits(iso.coords(), o["coords"])


def test_bad_connection_index_is_an_error(kvsmc_ctx):
    xyz, conn = cm.grid(1, 6, 6, 6, seed=1)
    v = cm.sphere_values(xyz)
    bad = conn.copy()
    bad[7, 3] = xyz.shape[0]          # one past the last node
    with pytest.raises(_abi.KvsmcError, match="connection index"):
        _abi.marching_cells_host(kvsmc_ctx, 1, v, xyz, bad, 1.5)
    # with a preset min/max the count pass finds it
    with pytest.raises(_abi.KvsmcError, match="connection index"):
        _abi.marching_cells_host(kvsmc_ctx, 1, v, xyz, bad, 1.5, (0.0, 5.0))
    # the context stays usable
    c, n, s = _abi.marching_cells_host(kvsmc_ctx, 1, v, xyz, conn, 1.5)
    assert same_bits(c, ocells.marching_cells(1, v, xyz, conn, 1.5)["coords"])


def test_device_entry_point_and_capacity(kvsmc_ctx):
    """kvsmc_marching_cells_device on torch device arrays: the same bits as the
    host call; too small outputs are KVSMC_ERR_CAPACITY with the sizes and
    nothing written."""
    import ctypes as C
    xyz, conn = cm.grid(3, 30, 28, 26, seed=11)
    v = cm.sphere_values(xyz, (14.2, 13.1, 12.6))
    dv, dx, dk = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (v, xyz, conn.view(np.int32)))
    torch.cuda.synchronize()
    s = _abi.Sizes()
    lib = kvsmc_ctx.lib

    def call(oc, cap_c, on, cap_n):
        return lib.kvsmc_marching_cells_device(kvsmc_ctx.handle, 3, dv.data_ptr(), 8, v.size, dx.data_ptr(),
                                               dk.data_ptr(), conn.shape[0], 6.5, 0, 0.0, 0.0, oc, cap_c, on, cap_n,
                                               C.byref(s))

    assert call(None, 0, None, 0) == 6          # KVSMC_ERR_CAPACITY
    t = s.ntriangles
    o = ocells.marching_cells(3, v, xyz, conn, 6.5)
    assert 9 * t == o["coords"].size > 0 and (s.min_value, s.max_value) == (o["vmin"], o["vmax"])
    oc = torch.full((9 * t,), 7.0, device="cuda")
    on = torch.full((3 * t,), 7.0, device="cuda")
    torch.cuda.synchronize()
    assert call(oc.data_ptr(), 9 * t - 1, on.data_ptr(), 3 * t) == 6
    assert bool((oc == 7.0).all())
    assert call(oc.data_ptr(), 9 * t, on.data_ptr(), 3 * t) == 0
    kvsmc_ctx.synchronize()
    assert same_bits(oc.cpu().numpy(), o["coords"]) and same_bits(on.cpu().numpy(), o["normals"])


def test_vertex_certificate_selftest(kvsmc_ctx):
    """The FP32 certificate of the cells' vertices never disagrees with the
    reference's FP64 sequence on adversarial random edges (close values,
    ratios at 0, 1/2, 1, large and tiny coordinates, coordinates crossing
    zero, equal endpoints), and decides most of them (exact midpoints, as
    c0 + d/2, are left to FP64 by design)."""
    for seed in (1, 2, 3):
        tested, mism, fall = kvsmc_ctx.selftest_cells(1 << 22, seed)
        assert tested > (1 << 21)
        assert mism == 0, (seed, mism)
        assert fall < 0.12 * tested, (seed, fall, tested)


def test_fast_and_exact_vertices_agree_on_adversarial_meshes(kvsmc_ctx):
    """Meshes built to land vertices near float rounding boundaries: integer
    values with isolevels at k + 1/2 (ratios 1/2) on power-of-two coordinates,
    and a preset min/max that clamps values."""
    rng = np.random.default_rng(17)
    for ct in range(4):
        xyz, conn = cm.grid(ct, 24, 20, 18, jitter=0.0, seed=ct)
        xyz = (xyz * np.float32(0.125) + np.float32(1024.0)).astype(np.float32)
        for dt, iso in ((np.uint8, 100.5), (np.int16, -3.5), (np.float32, 0.5)):
            v = rng.integers(0, 200, xyz.shape[0]).astype(dt) if dt is np.uint8 else (
                rng.integers(-10, 10, xyz.shape[0]).astype(dt) if dt is np.int16
                else (rng.integers(0, 2, xyz.shape[0]).astype(np.float32)))
            for mm in (None, (float(v.min()) + 1, float(v.max()) - 1)):
                c, n, s = _abi.marching_cells_host(kvsmc_ctx, ct, v, xyz, conn, iso, mm)
                o = ocells.marching_cells(ct, v, xyz, conn, iso, mm)
                assert same_bits(c, o["coords"]), (ct, dt, mm, first_diff(c, o["coords"]))
                assert same_bits(n, o["normals"]), (ct, dt, mm)


def test_bounds_match_the_fold_on_nans_and_signed_zeros(kvsmc_ctx):
    """kvsmc_cells_bounds against the restated fold (oracle/cells.py
    min_max_coords, itself pinned on the reference fixtures): NaN
    coordinates in the middle, at the very end and at the start, signed
    zeros tied with each other, with and without connections, and a large
    mesh."""
    rng = np.random.default_rng(23)
    for trial in range(24):
        ct = trial % 4
        xyz, conn = cm.random_mesh(ct, 400, 700, seed=trial)
        if trial % 3 == 0:
            xyz[rng.choice(400, 5, replace=False), rng.integers(0, 3, 5)] = np.nan
        if trial % 4 == 1:
            xyz[:, 1] = np.where(rng.random(400) < 0.5, np.float32(-0.0), np.float32(0.0))
        if trial % 5 == 2:
            xyz[conn.reshape(-1)[-1], 2] = np.nan          # the fold ends on a NaN
        if trial % 7 == 3:
            xyz[conn.reshape(-1)[0], 0] = np.nan           # the start is a NaN
        k = conn if trial % 6 != 5 else np.zeros((0, cm.NODES[ct]), np.uint32)
        lo, hi = _abi.cells_bounds(kvsmc_ctx, ct, xyz, k)
        wlo, whi = ocells.min_max_coords(xyz, k)
        assert same_bits(lo, wlo) and same_bits(hi, whi), (trial, lo, wlo, hi, whi)
    xyz, conn = cm.grid(0, 96, 96, 96, seed=3)
    lo, hi = _abi.cells_bounds(kvsmc_ctx, 0, xyz, conn)
    wlo, whi = ocells.min_max_coords(xyz, conn)
    assert same_bits(lo, wlo) and same_bits(hi, whi)


def test_isolevel_sweep_matches_single_extractions(kvsmc_ctx):
    """kvsmc_marching_cells_sweep_device: one count pass for all isolevels,
    the same bits per isolevel as kvsmc_marching_cells_device (and the
    restatement), every cell type, with and without a preset min/max; too
    small an output refuses the whole sweep with the sizes filled."""
    import ctypes as C
    lib = kvsmc_ctx.lib
    for ct in range(4):
        xyz, conn = cm.grid(ct, 40, 36, 32, seed=70 + ct)
        v = cm.sphere_values(xyz, (19.2, 17.4, 15.9))
        dv, dx, dk = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (v, xyz, conn.view(np.int32)))
        torch.cuda.synchronize()
        isos = [2.5 + 1.7 * i for i in range(12)]
        for mm in (None, (1.0, 20.0)):
            want = [ocells.marching_cells(ct, v, xyz, conn, iso, mm) for iso in isos]
            n = len(isos)
            caps = [max(1, w["coords"].size // 9) for w in want]
            oc = [torch.full((9 * c,), 7.0, device="cuda") for c in caps]
            on = [torch.full((3 * c,), 7.0, device="cuda") for c in caps]
            torch.cuda.synchronize()
            pc = (C.c_void_p * n)(*[t.data_ptr() for t in oc])
            pn = (C.c_void_p * n)(*[t.data_ptr() for t in on])
            cc = (C.c_uint64 * n)(*[9 * c for c in caps])
            cn = (C.c_uint64 * n)(*[3 * c for c in caps])
            sizes = (_abi.Sizes * n)()
            il = (C.c_double * n)(*isos)
            st = lib.kvsmc_marching_cells_sweep_device(
                kvsmc_ctx.handle, ct, dv.data_ptr(), 8, v.size, dx.data_ptr(), dk.data_ptr(), conn.shape[0], il, n,
                1 if mm else 0, mm[0] if mm else 0.0, mm[1] if mm else 0.0, pc, cc, pn, cn, sizes)
            assert st == 0, kvsmc_ctx.lib.kvsmc_last_error(kvsmc_ctx.handle)
            kvsmc_ctx.synchronize()
            for i, w in enumerate(want):
                t = sizes[i].ntriangles
                assert 9 * t == w["coords"].size, (ct, i)
                assert same_bits(oc[i][:9 * t].cpu().numpy(), w["coords"]), (ct, mm, i)
                assert same_bits(on[i][:3 * t].cpu().numpy(), w["normals"]), (ct, mm, i)
            # one output one triangle short: nothing written, sizes returned
            big = max(range(n), key=lambda i: caps[i])
            cc[big] = 9 * caps[big] - 9
            for t in oc:
                t.fill_(7.0)
            torch.cuda.synchronize()
            st = lib.kvsmc_marching_cells_sweep_device(
                kvsmc_ctx.handle, ct, dv.data_ptr(), 8, v.size, dx.data_ptr(), dk.data_ptr(), conn.shape[0], il, n,
                1 if mm else 0, mm[0] if mm else 0.0, mm[1] if mm else 0.0, pc, cc, pn, cn, sizes)
            assert st == 6 and sizes[big].ntriangles == caps[big]
            kvsmc_ctx.synchronize()
            assert all(bool((t == 7.0).all()) for t in oc)


def test_isolevel_sweep_on_random_meshes_with_ties(kvsmc_ctx):
    """The sweep on random connectivity (every table case, pyramid ambiguities
    with E == 0) with small integer values and isolevels on and between them."""
    import ctypes as C
    lib = kvsmc_ctx.lib
    rng = np.random.default_rng(31)
    for ct in range(4):
        xyz, conn = cm.random_mesh(ct, 3000, 60000, seed=200 + ct)
        v = rng.integers(-3, 4, 3000).astype(np.int16)
        isos = [-2.5, -1.0, 0.0, 0.5, 1.0, 2.0, 2.5]
        n = len(isos)
        want = [ocells.marching_cells(ct, v, xyz, conn, iso) for iso in isos]
        dv, dx, dk = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (v, xyz, conn.view(np.int32)))
        caps = [max(1, w["coords"].size // 9) for w in want]
        oc = [torch.empty(9 * c, device="cuda") for c in caps]
        on = [torch.empty(3 * c, device="cuda") for c in caps]
        torch.cuda.synchronize()
        sizes = (_abi.Sizes * n)()
        st = lib.kvsmc_marching_cells_sweep_device(
            kvsmc_ctx.handle, ct, dv.data_ptr(), 1, v.size, dx.data_ptr(), dk.data_ptr(), conn.shape[0],
            (C.c_double * n)(*isos), n, 0, 0.0, 0.0, (C.c_void_p * n)(*[t.data_ptr() for t in oc]),
            (C.c_uint64 * n)(*[9 * c for c in caps]), (C.c_void_p * n)(*[t.data_ptr() for t in on]),
            (C.c_uint64 * n)(*[3 * c for c in caps]), sizes)
        assert st == 0
        kvsmc_ctx.synchronize()
        for i, w in enumerate(want):
            t = sizes[i].ntriangles
            assert 9 * t == w["coords"].size, (ct, isos[i])
            assert same_bits(oc[i][:9 * t].cpu().numpy(), w["coords"]), (ct, isos[i])
            assert same_bits(on[i][:3 * t].cpu().numpy(), w["normals"]), (ct, isos[i])
