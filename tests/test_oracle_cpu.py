"""The oracle (oracle/mc_oracle.c) against the reference: the committed golden
fixtures (made from the reference build) and, where the reference sources are
present, the reference itself compiled from them (oracle/_ref)."""
import numpy as np
import pytest

from oracle import ref
from kvs_gb300 import synthetic as S

from .helpers import first_diff, golden, golden_inputs, golden_outputs, same_bits


def _oracle_run(oracle_lib, e, v, rect, cmap):
    obj = (e["obj"][0], e["obj"][1]) if e["obj"] else None
    return oracle_lib.marching_cubes(v, e["iso"], e["normal_type"], e["duplication"],
                                     minmax=tuple(e["minmax"]) if e["minmax"] else None,
                                     rect_coords=rect, obj_coords=obj, colormap=cmap,
                                     tf_range=tuple(e["tf_range"]) if e["tf_range"] else None)


def test_oracle_matches_golden_fixtures(oracle_lib):
    man, arr = golden()
    cmap = arr["colormap256"]
    assert len(man) > 800
    for e in man:
        v, rect = golden_inputs(e, arr)
        g = golden_outputs(e, arr)
        o = _oracle_run(oracle_lib, e, v, rect, cmap)
        tag = e["key"]
        assert o["success"] == e["success"], tag
        assert same_bits(o["coords"], g["coords"]), (tag, first_diff(o["coords"], g["coords"]))
        assert same_bits(o["normals"], g["normals"]), (tag, first_diff(o["normals"], g["normals"]))
        assert np.array_equal(o["connections"], g["connections"]), tag
        if g["coords"].size and np.isfinite(e["vol_min"]):
            assert np.array_equal(o["color"], g["colors"]), tag
        assert same_bits(np.array([o["vol_min"], o["vol_max"]]), np.array([e["vol_min"], e["vol_max"]])), tag
        assert np.array_equal(o["min_obj"], np.array(e["min_obj"], np.float32)), tag
        assert np.array_equal(o["max_obj"], np.array(e["max_obj"], np.float32)), tag


def test_oracle_colour_matches_golden(oracle_lib):
    _, arr = golden()
    import ctypes as C
    lib = oracle_lib.lib()
    t = np.ascontiguousarray(arr["colormap256"])
    for v, want in zip(arr["color_at_values"], arr["color_at_rgb"]):
        rgb = np.zeros(3, np.uint8)
        lib.mco_color_at(t.ctypes.data, 256, C.c_float(-1.0), C.c_float(2.0), C.c_float(float(v)), rgb.ctypes.data)
        assert np.array_equal(rgb, want), (v, rgb, want)


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference build (oracle/_ref) not present")


@needs_ref
@pytest.mark.parametrize("dtype", ref.DTYPES, ids=[np.dtype(d).name for d in ref.DTYPES])
def test_oracle_matches_reference_live(oracle_lib, dtype):
    rng = np.random.default_rng(hash(np.dtype(dtype).name) % 1000)
    cmap = ref.default_colormap(256)
    for shape in [(2, 2, 2), (5, 7, 9), (17, 13, 11), (3, 1, 8)]:
        if np.dtype(dtype).kind == "f":
            v = rng.random(shape).astype(dtype)
            isos = [0.5, 0.25, float(np.float32(0.3)), 0.1 + 1e-13]
        else:
            info = np.iinfo(dtype)
            lo, hi = max(int(info.min), -100), min(int(info.max), 100)
            v = rng.integers(lo, hi, size=shape, endpoint=True).astype(dtype)
            isos = [0.5, 3.0, -2.5, 17.0]
        for iso in isos:
            for nt, dup in [("polygon", True), ("polygon", False), ("vertex", True)]:
                a = ref.marching_cubes(v, iso, nt, dup)
                b = oracle_lib.marching_cubes(v, iso, nt, dup, colormap=cmap)
                tag = (shape, iso, nt, dup)
                assert same_bits(a["coords"], b["coords"]), tag
                assert same_bits(a["normals"], b["normals"]), tag
                assert np.array_equal(a["connections"], b["connections"]), tag
                if a["coords"].size:
                    assert np.array_equal(a["colors"], b["color"]), tag


@needs_ref
def test_oracle_matches_reference_on_workload_fields(oracle_lib):
    """The 128^3 blob workload and Hydrogen 64^3 (the reference example)."""
    v = S.to_numpy(S.gaussian_blobs((128, 128, 128), seed=42))
    a = ref.marching_cubes(v, 0.5)
    b = oracle_lib.marching_cubes(v, 0.5)
    assert a["coords"].size > 100000
    assert same_bits(a["coords"], b["coords"]) and same_bits(a["normals"], b["normals"])
    h = ref.hydrogen(64)
    iso = (float(h.min()) + float(h.max())) / 2
    for nt, dup in [("polygon", True), ("polygon", False), ("vertex", True)]:
        a = ref.marching_cubes(h, iso, nt, dup)
        b = oracle_lib.marching_cubes(h, iso, nt, dup)
        assert same_bits(a["coords"], b["coords"]) and same_bits(a["normals"], b["normals"])
        assert np.array_equal(a["connections"], b["connections"])
    assert ref.marching_cubes(h, iso)["coords"].size // 9 == 5680


@needs_ref
def test_oracle_matches_reference_edge_options(oracle_lib):
    rng = np.random.default_rng(77)
    v = rng.random((8, 9, 10)).astype(np.float32)
    cmap = ref.default_colormap(256)
    rect = np.concatenate([np.linspace(0, 3, 10), np.linspace(-1, 1, 9), np.linspace(2, 5, 8)]).astype(np.float32)
    for opts in [dict(minmax=(0.3, 0.7)), dict(minmax=(0.5, 0.5000001)), dict(obj_coords=([1, 2, 3], [4, 5, 6.5])),
                 dict(rect_coords=rect), dict(tf_range=(-2.0, 5.0))]:
        for nt, dup in [("polygon", True), ("polygon", False), ("vertex", True)]:
            a = ref.marching_cubes(v, 0.5, nt, dup, **opts)
            b = oracle_lib.marching_cubes(v, 0.5, nt, dup, colormap=cmap, **opts)
            assert same_bits(a["coords"], b["coords"]), opts
            assert same_bits(a["normals"], b["normals"]), opts
            assert np.array_equal(a["connections"], b["connections"]), opts
            if a["coords"].size:
                assert np.array_equal(a["colors"], b["color"]), opts


def test_checksum_mode_matches_the_stored_outputs(oracle_lib):
    """mco_dup_checksum (the oracle's loop folded into per-chunk checksums over
    a z-range) gives the counts and sums of the stored duplicated output, and a
    volume's slabs add up to the whole, so large outputs can be checked by sums."""
    import numpy as np
    from kvs_gb300 import synthetic as S
    v = S.to_numpy(S.gaussian_blobs((40, 48, 56), seed=3))
    lo, hi = float(v.min()), float(v.max())
    o = oracle_lib.extract(v, 0.5, 0, lo, hi, min_coord=(1.5, -2.0, 0.25), scale=(0.5, 2.0, 1.0))
    T = o["coords"].size // 9
    t, cs, ns = oracle_lib.dup_checksum(v, 0.5, lo, hi, min_coord=(1.5, -2.0, 0.25), scale=(0.5, 2.0, 1.0),
                                        chunk_tris=1000)
    assert t == T > 3000
    assert np.array_equal(cs, oracle_lib.mix_checksum(o["coords"], 9000))
    assert np.array_equal(ns, oracle_lib.mix_checksum(o["normals"], 3000))
    t0, c0, n0 = oracle_lib.dup_checksum(v, 0.5, lo, hi, 0, 17, min_coord=(1.5, -2.0, 0.25),
                                         scale=(0.5, 2.0, 1.0), chunk_tris=1 << 30)
    t1, c1, n1 = oracle_lib.dup_checksum(v, 0.5, lo, hi, 17, 39, min_coord=(1.5, -2.0, 0.25),
                                         scale=(0.5, 2.0, 1.0), chunk_tris=1 << 30)
    assert t0 + t1 == T
    assert np.array_equal(c0, oracle_lib.mix_checksum(o["coords"][:9 * t0], 9 << 30))
    assert np.array_equal(c1, oracle_lib.mix_checksum(o["coords"][9 * t0:], 9 << 30))
    assert np.array_equal(n1, oracle_lib.mix_checksum(o["normals"][3 * t0:], 3 << 30))
    # a changed bit or two swapped triangles change the sums
    bad = o["coords"].copy()
    bad.view(np.uint32)[5] ^= 1
    assert not np.array_equal(cs, oracle_lib.mix_checksum(bad, 9000))
    sw = o["coords"].reshape(-1, 9).copy()
    sw[[10, 11]] = sw[[11, 10]]
    assert not np.array_equal(cs, oracle_lib.mix_checksum(sw.ravel(), 9000))
