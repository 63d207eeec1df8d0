"""Generate the golden fixtures from the reference kvs::MarchingCubes and
kvs::Isosurface.

Runs the reference mappers compiled from their own sources (oracle/_ref, built
by oracle/Makefile.ref) on small seeded inputs and stores inputs + outputs in
tests/golden/golden.npz (case list tests/golden/cases.json) and
tests/golden/isosurface.npz (tests/golden/isosurface.json), and binary STL
files written by the reference PolygonExporter<kvs::Stl> in tests/golden/stl.npz
(tests/golden/stl.json), kvs::SlicePlane results in tests/golden/slice.npz
(tests/golden/slice.json), and the unstructured marching mappers
(MarchingTetrahedra / Hexahedra / Pyramid / Prism, directly and through
kvs::Isosurface) in tests/golden/cells.npz (tests/golden/cells.json), and
kvs::SlicePlane on unstructured volumes in tests/golden/slice_cells.npz
(tests/golden/slice_cells.json), and binary PLY files written by the reference
PolygonExporter<kvs::Ply> in tests/golden/ply.npz (tests/golden/ply.json), and the
reference's ASCII STL and KVSML polygon files (each writing data type) of
MarchingCubes results in tests/golden/exports.npz (tests/golden/exports.json).  The reference
ships no tests or golden vectors of its own, so these fixtures pin the oracle
restatement and the CUDA path on hosts where the reference is absent.

    python tests/golden/make_golden.py [marching_cubes] [isosurface] [stl] [slice] [cells] [slice_cells] [ply]
                                       [exports]
        (default: all)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from tests import cell_meshes as cm  # noqa: E402

MODES = [("polygon", True), ("polygon", False), ("vertex", True)]


def cases():
    rng = np.random.default_rng(2024)
    out = []
    h = ref.hydrogen(32)
    out.append(("hydrogen32", h, [(float(h.min()) + float(h.max())) / 2], {}))
    for dt in ref.DTYPES:
        dt = np.dtype(dt)
        if dt.kind == "f":
            v = rng.random((9, 10, 11)).astype(dt)
            isos = [0.5, float(np.float32(0.37))]
        else:
            info = np.iinfo(dt)
            lo, hi = max(int(info.min), -100), min(int(info.max), 100)
            v = rng.integers(lo, hi, size=(9, 10, 11), endpoint=True).astype(dt)
            isos = [0.5, 7.0]
        out.append((f"random_{dt.name}", v, isos, {}))
    x, y, z = np.meshgrid(np.arange(26), np.arange(24), np.arange(22), indexing="xy")
    blob = np.exp(-((x - 12.3) ** 2 + (y - 11.1) ** 2 + (z - 10.7) ** 2) / (2 * 6.0 ** 2)).transpose(2, 0, 1)
    blob = np.ascontiguousarray(blob).astype(np.float32)
    out.append(("blob_f32", blob, [0.5, 0.123456789], {}))
    f = rng.random((8, 9, 10)).astype(np.float32)
    out.append(("clamp_f32", f, [0.5], {"minmax": (0.3, 0.7)}))
    out.append(("objcoords_f32", f, [0.5], {"obj": ([1.5, -2.0, 3.25], [7.0, 9.0, 4.0])}))
    rect = np.concatenate([np.linspace(0, 3, 10), np.linspace(-1, 1, 9), np.linspace(2, 5, 8)]).astype(np.float32)
    out.append(("rectilinear_f32", f, [0.5], {"rect": rect}))
    out.append(("tfrange_f32", f, [0.5], {"tf_range": (-1.0, 3.0)}))
    out.append(("thin_x1_f32", rng.random((5, 6, 1)).astype(np.float32), [0.5], {}))
    out.append(("constant_f32", np.full((4, 5, 6), 2.0, np.float32), [2.0], {}))
    w = f.copy()
    w[3, 4, 5] = np.nan
    w[0, 0, 1] = -0.0
    out.append(("nan_f32", w, [0.5], {}))
    odd = rng.integers(0, 255, size=(6, 7, 33)).astype(np.uint8)
    out.append(("odd_u8", odd, [127.5, 100.0], {}))
    return out


def isosurface_cases():
    """(name, volume, [(form, isolevel, normal_type, duplication, minmax, tf_range), ...])"""
    rng = np.random.default_rng(77)
    h = ref.hydrogen(32)
    x, y, z = np.meshgrid(np.arange(26), np.arange(24), np.arange(22), indexing="xy")
    blob = np.exp(-((x - 12.3) ** 2 + (y - 11.1) ** 2 + (z - 10.7) ** 2) / (2 * 6.0 ** 2)).transpose(2, 0, 1)
    blob = np.ascontiguousarray(blob).astype(np.float32)
    f = rng.random((9, 10, 11)).astype(np.float32)
    w = f.copy()
    w[2, 3, 4] = np.nan
    return [
        ("hydrogen32", h, [(0, 0.0, "polygon", True, None, None), (0, 0.0, "vertex", True, None, None),
                           (1, 100.5, "polygon", True, None, None), (1, 100.5, "vertex", True, None, None),
                           (2, 60.0, "polygon", False, None, (0.0, 200.0)), (2, 60.0, "polygon", True, None, None)]),
        ("blob_f32", blob, [(0, 0.0, "polygon", True, None, None), (1, 0.3, "vertex", True, None, None),
                            (2, 0.5, "polygon", False, None, None)]),
        ("random_i16", rng.integers(-300, 300, (9, 10, 11)).astype(np.int16), [(0, 0.0, "polygon", True, None, None)]),
        ("random_u16", rng.integers(0, 60000, (6, 7, 33)).astype(np.uint16), [(0, 0.0, "polygon", True, None, None)]),
        ("random_f64", rng.random((9, 10, 11)), [(0, 0.0, "polygon", True, None, None),
                                                 (2, 0.5, "vertex", True, None, None)]),
        ("constant_f32", np.full((4, 5, 6), 2.0, np.float32), [(0, 0.0, "polygon", True, None, None)]),
        ("nan_f32", w, [(0, 0.0, "polygon", True, None, None)]),
        ("preset_f32", f, [(0, 0.0, "polygon", True, (0.2, 0.6), None), (1, 0.5, "polygon", True, (0.2, 0.6), None)]),
    ]


def write_isosurface():
    arrays, manifest = {}, []
    for name, v, runs in isosurface_cases():
        arrays[f"{name}__input"] = v
        for i, (form, iso, nt, dup, minmax, tfr) in enumerate(runs):
            key = f"{name}__{i}"
            r = ref.isosurface(v, form, iso, nt, dup, minmax=minmax, tf_range=tfr)
            for fld in ("coords", "normals", "connections", "colors", "opacities"):
                arrays[f"{key}__{fld}"] = r[fld]
            manifest.append(dict(key=key, case=name, form=form, isolevel=iso, normal_type=nt, duplication=dup,
                                 minmax=minmax, tf_range=tfr, success=r["success"], vol_min=r["vol_min"],
                                 vol_max=r["vol_max"], polygon_type=r["polygon_type"],
                                 normal_type_out=r["normal_type"], color_type=r["color_type"],
                                 min_obj=r["min_obj"].tolist(), max_obj=r["max_obj"].tolist(),
                                 min_ext=r["min_ext"].tolist(), max_ext=r["max_ext"].tolist()))
    np.savez_compressed(os.path.join(HERE, "isosurface.npz"), **arrays)
    with open(os.path.join(HERE, "isosurface.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} isosurface cases")


def stl_cases():
    """(name, volume, isolevel, normal_type, duplication) for the binary STL fixtures."""
    rng = np.random.default_rng(88)
    h = ref.hydrogen(32)
    x, y, z = np.meshgrid(np.arange(20), np.arange(18), np.arange(16), indexing="xy")
    blob = np.exp(-((x - 9.3) ** 2 + (y - 8.1) ** 2 + (z - 7.7) ** 2) / (2 * 5.0 ** 2)).transpose(2, 0, 1)
    blob = np.ascontiguousarray(blob).astype(np.float32)
    noise = rng.integers(0, 255, (9, 10, 11)).astype(np.uint8)
    return [
        ("hydrogen32_dup", h, 100.5, "polygon", True),
        ("hydrogen32_shared", h, 100.5, "polygon", False),
        ("hydrogen32_vertex", h, 100.5, "vertex", False),
        ("blob_f32_dup", blob, 0.5, "polygon", True),
        ("blob_f32_vertex", blob, 0.37, "vertex", True),
        ("noise_u8_dup", noise, 127.5, "polygon", True),
        ("noise_u8_vertex", noise, 127.5, "vertex", False),
        ("constant_f32", np.full((4, 5, 6), 2.0, np.float32), 2.0, "polygon", True),
    ]


def write_stl():
    arrays, manifest = {}, []
    for name, v, iso, nt, dup in stl_cases():
        arrays[f"{name}__input"] = v
        r = ref.marching_cubes(v, iso, nt, dup)
        for fld in ("coords", "normals", "connections"):
            arrays[f"{name}__{fld}"] = r[fld]
        arrays[f"{name}__stl"] = np.frombuffer(ref.marching_cubes_stl(v, iso, nt, dup), np.uint8)
        manifest.append(dict(case=name, isolevel=iso, normal_type=nt, duplication=dup,
                             normal_type_out=r["normal_type"], ntriangles=int(arrays[f"{name}__stl"][80:84].view("<u4")[0])))
    np.savez_compressed(os.path.join(HERE, "stl.npz"), **arrays)
    with open(os.path.join(HERE, "stl.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} stl cases")


def export_cases():
    """(name, volume, isolevel, normal_type, duplication) for the ASCII STL and
    KVSML fixtures: the reference's MarchingCubes result written by its own
    writers (kvsref_marching_cubes_export)."""
    h = ref.hydrogen(24)
    x, y, z = np.meshgrid(np.arange(12), np.arange(11), np.arange(10), indexing="xy")
    blob = np.exp(-((x - 5.3) ** 2 + (y - 5.1) ** 2 + (z - 4.7) ** 2) / (2 * 3.0 ** 2)).transpose(2, 0, 1)
    blob = np.ascontiguousarray(blob).astype(np.float32)
    # coordinates far from the origin: six-decimal rounding with long integer parts, negative normals
    big = np.ascontiguousarray(blob * np.float32(3.0) - np.float32(1.0))
    return [
        ("hydrogen24_dup", h, 100.5, "polygon", True),
        ("hydrogen24_vertex", h, 100.5, "vertex", False),
        ("hydrogen24_shared", h, 100.5, "polygon", False),
        ("blob12_dup", blob, 0.5, "polygon", True),
        ("blob12_vertex", blob, 0.37, "vertex", True),
        ("blob12_scaled", big, 0.61, "polygon", True),
        ("constant", np.full((4, 5, 6), 2.0, np.float32), 2.0, "polygon", True),
    ]


def write_exports():
    """Files of the reference's ASCII STL writer and of its KVSML polygon
    writer with each writing data type, as bytes, in tests/golden/exports.npz."""
    import tempfile
    arrays, manifest = {}, []
    with tempfile.TemporaryDirectory() as tmp:
        for name, v, iso, nt, dup in export_cases():
            arrays[f"{name}__input"] = v
            entry = dict(case=name, isolevel=iso, normal_type=nt, duplication=dup, files={})
            for fmt in ("stl_ascii", "kvsml_ascii", "kvsml_external_ascii", "kvsml_external_binary"):
                sub = os.path.join(tmp, fmt)
                os.makedirs(sub, exist_ok=True)
                main = os.path.join(sub, name + (".stl" if fmt.startswith("stl") else ".kvsml"))
                ref.marching_cubes_export(v, iso, nt, dup, fmt, main)
                files = sorted(f for f in os.listdir(sub) if f.startswith(name + ".") or f.startswith(name + "_"))
                entry["files"][fmt] = files
                for fn in files:
                    with open(os.path.join(sub, fn), "rb") as f:
                        arrays[f"{name}__{fmt}__{fn}"] = np.frombuffer(f.read(), np.uint8)
            manifest.append(entry)
    np.savez_compressed(os.path.join(HERE, "exports.npz"), **arrays)
    with open(os.path.join(HERE, "exports.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} export cases")


def slice_cases():
    """(name, volume, [(coefficients or None, point, normal, tf_range), ...])"""
    rng = np.random.default_rng(55)
    h = ref.hydrogen(16)
    x, y, z = np.meshgrid(np.arange(20), np.arange(18), np.arange(16), indexing="xy")
    blob = np.exp(-((x - 9.3) ** 2 + (y - 8.1) ** 2 + (z - 7.7) ** 2) / (2 * 5.0 ** 2)).transpose(2, 0, 1)
    blob = np.ascontiguousarray(blob).astype(np.float32)
    shape = (9, 10, 11)
    obl = (None, (5.3, 4.7, 3.9), (0.31, -0.52, 0.79), None)
    return [
        ("hydrogen16", h, [((0, 0, 1, -7.5), None, None, None), obl, ((0, 0, 1, -7), None, None, None),
                           ((1, 1, 1, -20), None, None, None), ((0, 0, 1, 100), None, None, None),
                           (None, (7.3, 7.7, 8.1), (0.3, -0.5, 0.8), (10.0, 200.0))]),
        ("blob_f32", blob, [obl, ((0.2, 0.9, -0.4, -3.3), None, None, None)]),
        ("random_i8", rng.integers(-128, 128, shape).astype(np.int8), [((0, 0, 1, -4.25), None, None, None)]),
        ("random_u16", rng.integers(0, 65536, shape).astype(np.uint16), [((1, 0, 0, -5.5), None, None, None)]),
        ("random_i16", rng.integers(-3000, 3000, shape).astype(np.int16), [obl]),
        ("random_i32", rng.integers(-2 ** 30, 2 ** 30, shape).astype(np.int32), [obl]),
        ("random_u32", rng.integers(0, 2 ** 32 - 1, shape, dtype=np.uint64).astype(np.uint32), [obl]),
        ("random_i64", rng.integers(-2 ** 60, 2 ** 60, shape).astype(np.int64), [obl]),
        ("random_u64", rng.integers(0, 2 ** 63, shape, dtype=np.uint64), [obl]),
        ("random_f64", rng.standard_normal(shape), [obl]),
        ("constant_f32", np.full((4, 5, 6), 2.0, np.float32), [((0, 1, 0, -1.5), None, None, None)]),
    ]


def write_slice():
    arrays, manifest = {}, []
    for name, v, runs in slice_cases():
        arrays[f"{name}__input"] = v
        for i, (coef, point, normal, tfr) in enumerate(runs):
            key = f"{name}__{i}"
            r = ref.slice_plane(v, coefficients=coef, point=point, normal=normal, tf_range=tfr)
            for fld in ("coords", "normals", "colors", "opacities"):
                arrays[f"{key}__{fld}"] = r[fld]
            manifest.append(dict(key=key, case=name, coefficients=coef, point=point, normal=normal, tf_range=tfr,
                                 success=r["success"], polygon_type=r["polygon_type"], color_type=r["color_type"],
                                 normal_type=r["normal_type"], min_obj=r["min_obj"].tolist(),
                                 max_obj=r["max_obj"].tolist(), min_ext=r["min_ext"].tolist(),
                                 max_ext=r["max_ext"].tolist(), ntriangles=int(r["coords"].size // 9)))
    np.savez_compressed(os.path.join(HERE, "slice.npz"), **arrays)
    with open(os.path.join(HERE, "slice.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} slice cases")


def cells_cases():
    """(name, cell_type, values, coords, connections, [run options, ...]); a run
    is dict(iso, form, normal_type, duplication, minmax, tf_range)."""
    out = []
    base = dict(form=0, normal_type="polygon", duplication=True, minmax=None, tf_range=None)

    def run(**kw):
        r = dict(base)
        r.update(kw)
        return r

    for ct, tag in ((0, "tet"), (1, "hex"), (2, "pyr"), (3, "pri")):
        seed = 100 + ct
        rng = np.random.default_rng(seed)
        xyz, conn = cm.grid(ct, 7, 6, 5, seed=seed)
        v = cm.sphere_values(xyz)
        out.append((f"{tag}_grid_f32", ct, v, xyz, conn,
                    [run(iso=1.7), run(iso=2.45), run(iso=1.7, normal_type="vertex"),
                     run(iso=1.7, duplication=False), run(iso=1.7, form=1), run(iso=2.0, tf_range=(0.5, 3.0)),
                     run(iso=1.7, minmax=(1.2, 2.2))]))
        xyz, conn = cm.random_mesh(ct, 120, (300, 120, 200, 160)[ct], seed=seed)
        n = xyz.shape[0]
        out.append((f"{tag}_random_f64", ct, rng.standard_normal(n), xyz, conn,
                    [run(iso=0.1), run(iso=-0.35, minmax=(-0.5, 0.5)), run(iso=0.1, form=1, duplication=False)]))
        small = rng.integers(-2, 3, n)
        out.append((f"{tag}_random_i8", ct, small.astype(np.int8), xyz, conn,
                    [run(iso=0.0), run(iso=0.5), run(iso=1.0)]))
        out.append((f"{tag}_random_u8", ct, rng.integers(0, 256, n).astype(np.uint8), xyz, conn,
                    [run(iso=100.5)]))
        out.append((f"{tag}_random_i16", ct, rng.integers(-3000, 3000, n).astype(np.int16), xyz, conn,
                    [run(iso=17.0)]))
        out.append((f"{tag}_random_u16", ct, rng.integers(0, 65536, n).astype(np.uint16), xyz, conn,
                    [run(iso=30000.25)]))
        out.append((f"{tag}_random_i32", ct, rng.integers(-2 ** 30, 2 ** 30, n).astype(np.int32), xyz, conn,
                    [run(iso=12345.5)]))
        out.append((f"{tag}_random_u32", ct, rng.integers(0, 2 ** 32 - 1, n, dtype=np.uint64).astype(np.uint32),
                    xyz, conn, [run(iso=2.0 ** 31)]))
        out.append((f"{tag}_random_i64", ct, rng.integers(-2 ** 60, 2 ** 60, n).astype(np.int64), xyz, conn,
                    [run(iso=3.0 ** 30)]))
        out.append((f"{tag}_random_u64", ct, rng.integers(0, 2 ** 63, n, dtype=np.uint64), xyz, conn,
                    [run(iso=2.0 ** 62)]))
        vn = rng.standard_normal(n).astype(np.float32)
        vn[rng.choice(np.arange(1, n), 6, replace=False)] = np.nan
        out.append((f"{tag}_nan_f32", ct, vn, xyz, conn, [run(iso=0.2)]))
        v0 = rng.standard_normal(n).astype(np.float32)
        v0[0] = np.nan
        # (a NaN min/max with no transfer-function range makes the reference
        # index its colour table with a NaN, undefined behaviour: give a range)
        out.append((f"{tag}_nan0_f32", ct, v0, xyz, conn, [run(iso=0.2, tf_range=(-1.0, 1.0))]))
        out.append((f"{tag}_constant_f32", ct, np.full(n, 1.5, np.float32), xyz, conn, [run(iso=1.5)]))
        # node 0 off the cells with the largest value (min/max scan starts there)
        conn1 = np.where(conn == 0, 1, conn).astype(np.uint32)
        vz = rng.standard_normal(n).astype(np.float32)
        vz[0] = 50.0
        out.append((f"{tag}_unref0_f32", ct, vz, xyz, conn1, [run(iso=0.3)]))
        # signed zeros: the first occurrence decides the sign of min/max
        vs = np.where(rng.random(n) < 0.5, np.float32(-0.0), np.float32(0.0)).astype(np.float32)
        vs[rng.choice(n, n // 3, replace=False)] = np.float32(1.0)
        out.append((f"{tag}_zeros_f32", ct, vs, xyz, conn, [run(iso=0.5), run(iso=0.0)]))
        # no cells: min/max over the nodes, nothing extracted
        out.append((f"{tag}_nocells_f32", ct, rng.standard_normal(n).astype(np.float32), xyz,
                    np.zeros((0, cm.NODES[ct]), np.uint32), [run(iso=0.0)]))
    return out


def write_cells():
    arrays, manifest = {}, []
    for name, ct, v, xyz, conn, runs in cells_cases():
        arrays[f"{name}__values"] = v
        arrays[f"{name}__coords"] = xyz
        arrays[f"{name}__connections"] = conn
        for i, o in enumerate(runs):
            key = f"{name}__{i}"
            r = ref.marching_cells(ct, v, xyz, conn, o["iso"], form=o["form"], normal_type=o["normal_type"],
                                   duplication=o["duplication"], minmax=o["minmax"], tf_range=o["tf_range"])
            for fld in ("coords", "normals", "connections", "colors", "opacities"):
                arrays[f"{key}__{fld}"] = r[fld]
            arrays[f"{key}__vol_minmax"] = np.array([r["vol_min"], r["vol_max"]], np.float64)
            manifest.append(dict(key=key, case=name, cell_type=ct, **{k: o[k] for k in o},
                                 success=r["success"], vol_has_minmax=r["vol_has_minmax"],
                                 polygon_type=r["polygon_type"], color_type=r["color_type"],
                                 normal_type_out=r["normal_type"], min_obj=r["min_obj"].tolist(),
                                 max_obj=r["max_obj"].tolist(), min_ext=r["min_ext"].tolist(),
                                 max_ext=r["max_ext"].tolist(), ntriangles=int(r["coords"].size // 9)))
    np.savez_compressed(os.path.join(HERE, "cells.npz"), **arrays)
    with open(os.path.join(HERE, "cells.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} cells cases")


def slice_cells_cases():
    """(name, cell_type, values, coords, connections, [run: dict(coefficients | point+normal, tf_range)])"""
    out = []
    obl = dict(coefficients=(0.31, -0.52, 0.79, -1.37))
    for ct, tag in ((0, "tet"), (1, "hex"), (2, "pyr"), (3, "pri")):
        seed = 300 + ct
        rng = np.random.default_rng(seed)
        xyz, conn = cm.grid(ct, 7, 6, 5, seed=seed)
        v = cm.sphere_values(xyz)
        out.append((f"{tag}_grid_f32", ct, v, xyz, conn,
                    [obl, dict(point=(2.9, 2.4, 1.7), normal=(0.3, -0.5, 0.8)), dict(coefficients=(1, 1, 1, -6.5)),
                     dict(coefficients=(0, 0, 1, 100)), dict(coefficients=(0.2, 0.9, -0.4, -1.1), tf_range=(1.0, 3.0))]))
        # nodes exactly on the plane (unjittered grid, plane z = 2 and x = 3)
        xyz0, conn0 = cm.grid(ct, 6, 5, 5, jitter=0.0, seed=seed)
        out.append((f"{tag}_flat_f32", ct, cm.sphere_values(xyz0), xyz0, conn0,
                    [dict(coefficients=(0, 0, 1, -2)), dict(coefficients=(1, 0, 0, -3))]))
        xyz, conn = cm.random_mesh(ct, 120, (300, 120, 200, 160)[ct], seed=seed)
        n = xyz.shape[0]
        for dt, gen in ((np.int8, lambda: rng.integers(-128, 128, n)), (np.uint8, lambda: rng.integers(0, 256, n)),
                        (np.int16, lambda: rng.integers(-3000, 3000, n)),
                        (np.uint16, lambda: rng.integers(0, 65536, n)),
                        (np.int32, lambda: rng.integers(-2 ** 30, 2 ** 30, n)),
                        (np.uint32, lambda: rng.integers(0, 2 ** 32 - 1, n, dtype=np.uint64)),
                        (np.int64, lambda: rng.integers(-2 ** 60, 2 ** 60, n)),
                        (np.uint64, lambda: rng.integers(0, 2 ** 63, n, dtype=np.uint64)),
                        (np.float64, lambda: rng.standard_normal(n))):
            out.append((f"{tag}_random_{np.dtype(dt).name}", ct, gen().astype(dt), xyz, conn, [obl]))
        out.append((f"{tag}_nocells_f32", ct, rng.standard_normal(n).astype(np.float32), xyz,
                    np.zeros((0, cm.NODES[ct]), np.uint32), [obl]))
    return out


def write_slice_cells():
    arrays, manifest = {}, []
    for name, ct, v, xyz, conn, runs in slice_cells_cases():
        arrays[f"{name}__values"] = v
        arrays[f"{name}__coords"] = xyz
        arrays[f"{name}__connections"] = conn
        for i, o in enumerate(runs):
            key = f"{name}__{i}"
            r = ref.slice_cells(ct, v, xyz, conn, coefficients=o.get("coefficients"), point=o.get("point"),
                                normal=o.get("normal"), tf_range=o.get("tf_range"))
            for fld in ("coords", "normals", "colors", "opacities"):
                arrays[f"{key}__{fld}"] = r[fld]
            arrays[f"{key}__vol_minmax"] = np.array([r["vol_min"], r["vol_max"]], np.float64)
            manifest.append(dict(key=key, case=name, cell_type=ct, coefficients=o.get("coefficients"),
                                 point=o.get("point"), normal=o.get("normal"), tf_range=o.get("tf_range"),
                                 success=r["success"], polygon_type=r["polygon_type"], color_type=r["color_type"],
                                 normal_type=r["normal_type"], min_obj=r["min_obj"].tolist(),
                                 max_obj=r["max_obj"].tolist(), max_ext=r["max_ext"].tolist(),
                                 ntriangles=int(r["coords"].size // 9)))
    np.savez_compressed(os.path.join(HERE, "slice_cells.npz"), **arrays)
    with open(os.path.join(HERE, "slice_cells.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} slice_cells cases")


_PLY_CHILD = """
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from oracle import ref
d = np.load(sys.argv[2])
ref.write_ply(sys.argv[3], d["coords"], d["colors"], d["normals"], str(d["color_type"]), str(d["normal_type"]))
"""


def ply_cases():
    """(name, coords, colors, normals, color_type, normal_type)"""
    rng = np.random.default_rng(91)
    blob = ref.marching_cubes(cases()[1][1], 0.45)          # a duplicated marching-cubes mesh, one colour
    sl = ref.slice_plane(ref.hydrogen(16), coefficients=(0.3, -0.5, 0.8, -4.0))   # vertex colours
    nv = 300
    return [
        ("mc_dup", blob["coords"], blob["colors"], blob["normals"], "polygon", "polygon"),
        ("slice", sl["coords"], sl["colors"], sl["normals"], "vertex", "polygon"),
        ("vertex_normals", rng.standard_normal(3 * nv).astype(np.float32), rng.integers(0, 256, 3 * nv).astype(np.uint8),
         rng.standard_normal(3 * nv).astype(np.float32), "vertex", "vertex"),
        ("bare", rng.standard_normal(3 * nv).astype(np.float32), np.zeros(0, np.uint8), np.zeros(0, np.float32),
         "polygon", "polygon"),
        ("one_colour_no_normals", rng.standard_normal(3 * nv).astype(np.float32), np.array([7, 8, 9], np.uint8),
         np.zeros(0, np.float32), "polygon", "polygon"),
        ("empty", np.zeros(0, np.float32), np.zeros(0, np.uint8), np.zeros(0, np.float32), "polygon", "polygon"),
    ]


def write_ply_fixtures():
    """The reference writer aborts while freeing its tables after closing the
    file (PlyFile.cpp:1345-1366), so each file is written by a child process
    and read back from disk."""
    import subprocess
    import tempfile
    arrays, manifest = {}, []
    with tempfile.TemporaryDirectory() as tmp:
        for name, c, k, n, ct, nt in ply_cases():
            inp = os.path.join(tmp, name + ".npz")
            out = os.path.join(tmp, name + ".ply")
            np.savez(inp, coords=c, colors=k, normals=n, color_type=ct, normal_type=nt)
            r = subprocess.run([sys.executable, "-c", _PLY_CHILD, ROOT, inp, out], capture_output=True)
            data = np.frombuffer(open(out, "rb").read(), np.uint8)
            arrays[f"{name}__coords"] = c
            arrays[f"{name}__colors"] = k
            arrays[f"{name}__normals"] = n
            arrays[f"{name}__file"] = data
            manifest.append(dict(case=name, color_type=ct, normal_type=nt, bytes=int(data.size),
                                 child_status=r.returncode))
    np.savez_compressed(os.path.join(HERE, "ply.npz"), **arrays)
    with open(os.path.join(HERE, "ply.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} ply cases")


def main():
    if not ref.available():
        ref.build()
    parts = sys.argv[1:] or ["marching_cubes", "isosurface", "stl", "slice", "cells", "slice_cells", "ply", "exports"]
    if "exports" in parts:
        write_exports()
    if "ply" in parts:
        write_ply_fixtures()
    if "cells" in parts:
        write_cells()
    if "slice_cells" in parts:
        write_slice_cells()
    if "slice" in parts:
        write_slice()
    if "isosurface" in parts:
        write_isosurface()
    if "stl" in parts:
        write_stl()
    if "marching_cubes" not in parts:
        return
    arrays = {}
    manifest = []
    for name, v, isos, opts in cases():
        arrays[f"{name}__input"] = v
        if "rect" in opts:
            arrays[f"{name}__rect"] = opts["rect"]
        for iso in isos:
            for nt, dup in MODES:
                key = f"{name}__{iso!r}__{nt}__{int(dup)}"
                r = ref.marching_cubes(v, iso, nt, dup, minmax=opts.get("minmax"), rect_coords=opts.get("rect"),
                                       obj_coords=opts.get("obj"), tf_range=opts.get("tf_range"))
                for f in ("coords", "normals", "connections", "colors"):
                    arrays[f"{key}__{f}"] = r[f]
                manifest.append(dict(key=key, case=name, iso=iso, normal_type=nt, duplication=dup,
                                     minmax=opts.get("minmax"), obj=opts.get("obj"), rect="rect" in opts,
                                     tf_range=opts.get("tf_range"), success=r["success"],
                                     vol_min=r["vol_min"], vol_max=r["vol_max"],
                                     polygon_type=r["polygon_type"], normal_type_out=r["normal_type"],
                                     color_type=r["color_type"], min_obj=r["min_obj"].tolist(),
                                     max_obj=r["max_obj"].tolist(), ntriangles=int(
                                         r["coords"].size // 9 if dup and nt == "polygon"
                                         else r["connections"].size // 3)))
    # every corner configuration, each in its own 2x2x2 volume
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for case in range(256):
        v = np.zeros((2, 2, 2), np.float32)
        for k, (x, y, z) in enumerate(corner):
            v[z, y, x] = 1.0 if case & (1 << k) else 0.0
        arrays[f"case{case}__input"] = v
        for nt, dup in MODES:
            key = f"case{case}__0.5__{nt}__{int(dup)}"
            r = ref.marching_cubes(v, 0.5, nt, dup)
            for f in ("coords", "normals", "connections", "colors"):
                arrays[f"{key}__{f}"] = r[f]
            manifest.append(dict(key=key, case=f"case{case}", iso=0.5, normal_type=nt, duplication=dup,
                                 minmax=None, obj=None, rect=False, tf_range=None, success=r["success"],
                                 vol_min=r["vol_min"], vol_max=r["vol_max"], polygon_type=r["polygon_type"],
                                 normal_type_out=r["normal_type"], color_type=r["color_type"],
                                 min_obj=r["min_obj"].tolist(), max_obj=r["max_obj"].tolist(), ntriangles=-1))
    # the default colour table and ColorMap::at on a sweep of values
    arrays["colormap256"] = ref.default_colormap(256)
    vals = np.linspace(-1.5, 2.5, 97).astype(np.float32)
    arrays["color_at_values"] = vals
    arrays["color_at_rgb"] = np.stack([ref.color_at(256, np.float32(-1.0), np.float32(2.0), v) for v in vals])
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(manifest, f, indent=0)
    print(f"{len(manifest)} golden cases")


if __name__ == "__main__":
    main()
