"""Benchmark: multi-isovalue marching-cubes sweep on one GB300.

Default workload (the headline configuration): a 1024^3 float32 field of
seeded 5-octave fBm gradient noise (base frequency 1/128, gain 0.5, rescaled
to [0, 1]), 16 isovalues 0.2 + 0.04 k, duplicated vertices + polygon normals.
A step is one kvsmc_extract_batch call over the 16 requests on the resident
volume: the fused count launch, the scan, the fused emit launch, with output
written to HBM.  `value` = cells x isovalues / s (Mcells/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload sweep1024|sweep512|uneven200|serve|heavy|stl512|stl384|kvsml512|slice1024|blobs128]
                    [--tune]

--tune runs the launch-shape autotuner (kvsmc_autotune, a few seconds) on the
bench's context before measuring; without it the built-in rules decide.

--workload serve runs the request loop (kvsmc_server_*) under Poisson
arrivals at each offered rate and reports p50/p99 latency and throughput.

--workload uneven200 times the same 200-request batch three ways: one plain
kvsmc_extract_device call per request (count, host sync, emit, host sync),
one kvsmc_extract_batch call, and one replay of a kvsmc_plan (the whole batch
captured in a CUDA graph); `value` is the plan replay.

--impl reference times the reference's CPU algorithm on this host's cores: the
C restatement under oracle/ (the reference sources are not present on the GPU
host), on a bounded slab sample of the same workload, all cores.
N > 1 (torchrun): independent replicas, one per GPU ("scaling": "weak").
"""
import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "sweep1024": dict(shape=(1024, 1024, 1024), kind="fbm", isos=[0.2 + 0.04 * k for k in range(16)],
                      desc="1024^3 float32 fBm gradient noise (5 octaves, base freq 1/128, gain 0.5, in [0,1]), "
                           "16 isovalues 0.2..0.8 in one batched call, duplication=true, PolygonNormal"),
    "sweep512": dict(shape=(512, 512, 512), kind="fbm", isos=[0.2 + 0.04 * k for k in range(16)],
                     desc="512^3 float32 fBm gradient noise (as sweep1024), 16 isovalues 0.2..0.8 in one batched "
                          "call, duplication=true, PolygonNormal (the profiling case: same kernel instance as "
                          "sweep1024)"),
    "uneven200": dict(kind="batch", n=200, dims=(32, 384), seed=2024,
                      desc="200 volumes, each axis U[32,384], dtype U{uint8,uint16,float32}, ellipsoid phantoms "
                           "(3-6 nested rotated shells + N(0, 2% range) noise), one isovalue per volume U over the "
                           "central 60% of its range, duplication=true, PolygonNormal"),
    "serve": dict(kind="serve", seed=77, rates=[100, 500, 2000], seconds=3.0,
                  volumes=[("fbm", (256, 256, 256), np.float32)] * 4 + [("phantom", (512, 512, 512), np.uint16)] * 2
                  + [("blobs", (768, 768, 768), np.float32)] * 2,
                  desc="serving loop: 8 resident volumes (4x 256^3 f32 fBm, 2x 512^3 u16 phantoms, 2x 768^3 f32 "
                       "Gaussian blobs); Poisson arrivals at 100, 500, 2000 req/s, each request a uniform volume and "
                       "an isovalue uniform in its 10th-90th value percentiles; 40 GiB output budget; "
                       "duplication=true, PolygonNormal"),
    "heavy": dict(shape=(1024, 2048, 2048), kind="lattice", spacing=48, dtype=np.uint16,
                  pcts=[0.45, 0.50, 0.55, 0.60],
                  desc="output-heavy stress: 2048x2048x1024 uint16, white noise U[0,65535] low-passed (lattice "
                       "spacing 48, trilinear; a 3-tap box filter leaves 1.64 triangles per cell per isovalue, "
                       "2.8e10 triangles / 1.3 TB for 4 isovalues, against the stated ~1e9), 4 isovalues at the "
                       "45/50/55/60th percentiles in one batched call (~1.1e9 triangles), duplication=true, "
                       "PolygonNormal"),
    "stl512": dict(shape=(512, 512, 512), kind="stl", isos=[0.2 + 0.04 * k for k in range(16)],
                   desc="binary STL serialisation on the GPU of the 16 duplicated-vertex meshes of the 512^3 "
                        "float32 fBm sweep (80 M triangles, 3.9 GB in, 4.0 GB of 50-byte records out per step); "
                        "e2e = kvsmc_write_stl of all 16 to /dev/null (GPU records, copy to pinned memory, fwrite)"),
    "stlascii512": dict(shape=(512, 512, 512), kind="stlascii", isos=[0.2 + 0.04 * k for k in range(16)],
                        desc="ASCII STL (the kvs::Stl default file type) of the 16 duplicated-vertex meshes of the "
                             "512^3 float32 fBm sweep, text formatted on the GPU (exact %f), copied to pinned memory "
                             "and written to /dev/null, kvsmc_write_stl_ascii per mesh"),
    "stl384": dict(shape=(384, 384, 384), kind="stl", isos=[0.2 + 0.04 * k for k in range(16)],
                   desc="binary STL serialisation of the 16 meshes of a 384^3 float32 fBm sweep (the profiling "
                        "case of stl512: same kernel, ~3.5 GB on the device, each launch larger than L2)"),
    "kvsml512": dict(shape=(512, 512, 512), kind="ingest",
                     desc="KVSML ingest: a 512^3 float32 structured volume (external binary, 512 MiB, page cache "
                          "under /dev/shm) loaded straight into a padded device volume by kvsmc_volume_load_kvsml "
                          "(header parse, chunked pinned reads + cudaMemcpy2DAsync, min/max scan, brick table)"),
    "slice1024": dict(shape=(1024, 1024, 1024), kind="slice", point=(511.5, 511.5, 511.5), normal=(0.31, -0.52, 0.79),
                      desc="kvs::SlicePlane of the 1024^3 float32 fBm field by the oblique plane through its "
                           "centre with normal (0.31, -0.52, 0.79): count + emit (coords, per-vertex colours from "
                           "the default colour map, normals) into device buffers through kvsmc_slice_extract_device"),
    "tet160": dict(kind="cells", n=161, radii=[30.0, 50.0, 70.0, 90.0], seed=9,
                   desc="kvs::MarchingTetrahedra on an unstructured volume: a 161^3-node grid (unit spacing, "
                        "nodes jittered U[-0.2,0.2]) split into 6 tetrahedra per hexahedron (24.6 M cells, 4.17 M "
                        "nodes), float32 values = distance to (80.3, 79.6, 80.9) + 1.5 sin(x/7) sin(y/9) sin(z/11), "
                        "one isolevel per step cycling 30/50/70/90, duplication=true, PolygonNormal"),
    "slice512": dict(shape=(512, 512, 512), kind="slice", point=(255.5, 255.5, 255.5), normal=(0.31, -0.52, 0.79),
                     desc="kvs::SlicePlane of a 512^3 float32 fBm field by the oblique plane through its centre "
                          "with normal (0.31, -0.52, 0.79) (the profiling case of slice1024: same kernels, "
                          "512 MiB on the device)"),
    "blobs128vn": dict(shape=(128, 128, 128), kind="blobs", isos=[0.5], mode=2,
                       desc="128^3 float32, 4 Gaussian blobs (sigma 8..24) + U[-0.01,0.01] noise, iso 0.5, "
                            "VertexNormal (shared vertices + connections + per-vertex normals: the mode of the "
                            "reference's own isosurface example)"),
    "sweep1024vn": dict(shape=(1024, 1024, 1024), kind="fbm", isos=[0.2 + 0.04 * k for k in range(16)], mode=2,
                        desc="1024^3 float32 fBm (as sweep1024), 16 isovalues 0.2..0.8 in one batched call, "
                             "VertexNormal (shared vertices + connections + per-vertex normals)"),
    "sweep512vn": dict(shape=(512, 512, 512), kind="fbm", isos=[0.2 + 0.04 * k for k in range(16)], mode=2,
                       desc="512^3 float32 fBm (as sweep1024), 16 isovalues, VertexNormal (the profiling case of "
                            "sweep1024vn: same kernels, 512 MiB on the device)"),
    "blobs128": dict(shape=(128, 128, 128), kind="blobs", isos=[0.5],
                     desc="128^3 float32, 4 Gaussian blobs (sigma 8..24) + U[-0.01,0.01] noise, iso 0.5, "
                          "duplication=true, PolygonNormal"),
}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value, world):
    """Max over ranks of a float (identity for one rank); NCCL or gloo."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ms_per_rank, world):
    """Whole-job throughput of independent replicas: all ranks' units over the
    slowest rank's time (units/s)."""
    return units_per_rank * world / (barrier_max(ms_per_rank, world) * 1e-3)


def make_field(w, device, seed=42):
    from kvs_gb300 import synthetic as S
    if w["kind"] == "fbm":
        return S.fbm(w["shape"], seed=seed, device=device)
    if w["kind"] == "lattice":
        return S.lattice_noise(w["shape"], w["dtype"], seed=seed, device=device, spacing=w["spacing"])
    return S.gaussian_blobs(w["shape"], seed=seed, device=device)


def workload_isos(w, sample):
    """The workload's isovalues: fixed, or percentiles of a value sample
    (a flat float64 array)."""
    if "pcts" in w:
        return [float(np.quantile(sample, q)) for q in w["pcts"]]
    return list(w["isos"])


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"kvsmc_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, val in zip(names, p[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(n)
            os.remove(self.path)
        except Exception:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch(workload):
    """DRAM bytes of one emit launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"stream_emit_{workload}.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("dram_bytes_per_launch")
    return None


# ----------------------------------------------------------------- our arm

def maybe_tune(args, ctx):
    """--tune: run the launch-shape autotuner on this context first; returns
    a summary for the JSON line (None without --tune)."""
    if not args.tune:
        return None
    import time

    from kvs_gb300 import autotune as T
    t0 = time.time()
    table = T.autotune(ctx, max_class=4, isovalues=4, reps=3)
    changed = [r for r in table if any(r[f] for f in T.FIELDS)]
    return {"seconds": round(time.time() - t0, 2), "entries": len(table), "entries_changed": len(changed),
            "changed": [{k: r[k] for k in ("dtype", "size_class") + T.FIELDS} for r in changed]}


def run_slice(args, rank, world, local):
    """kvsmc_slice_extract_device of one oblique plane through a 1024^3 field."""
    import ctypes as C

    import torch

    from kvs_gb300 import _abi
    from kvs_gb300.marching_cubes import TransferFunction

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    nz, ny, nx = w["shape"]
    field = make_field(dict(w, kind="fbm"), "cuda")
    torch.cuda.synchronize()
    vol = _abi.DeviceVolume.from_device(ctx, field.data_ptr(), np.float32, field.shape)
    del field
    torch.cuda.empty_cache()
    lo, hi = vol.minmax()
    pt, nrm = np.float32(w["point"]), np.float32(w["normal"])
    dot = np.float32(np.float32(np.float32(pt[0] * nrm[0]) + np.float32(pt[1] * nrm[1])) + np.float32(pt[2] * nrm[2]))
    table = np.ascontiguousarray(TransferFunction(256).table, np.uint8)
    p = _abi.SliceParams()
    for i, c in enumerate((nrm[0], nrm[1], nrm[2], -dot)):
        p.coefficients[i] = float(c)
    for i in range(3):
        p.min_coord[i], p.scale[i] = 0.0, 1.0
    p.tf_min, p.tf_max, p.tf_resolution, p.tf_table = float(lo), float(hi), 256, table.ctypes.data
    n = C.c_uint64(0)
    ctx.check(ctx.lib.kvsmc_slice_count(ctx.handle, vol.handle, C.byref(p), C.byref(n)), "slice_count")
    t = n.value
    c = torch.empty(max(1, 9 * t), dtype=torch.float32, device="cuda")
    k = torch.empty(max(1, 9 * t), dtype=torch.uint8, device="cuda")
    nn = torch.empty(max(1, 3 * t), dtype=torch.float32, device="cuda")

    def step():
        ctx.check(ctx.lib.kvsmc_slice_extract_device(ctx.handle, vol.handle, C.byref(p), c.data_ptr(), 9 * t,
                                                     k.data_ptr(), 9 * t, nn.data_ptr(), 3 * t, C.byref(n)),
                  "slice_extract_device")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ctx.profile_enable(True)
    launches0 = ctx.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = barrier_max(e0.elapsed_time(e1), world) / args.steps
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    cells = (nx - 1) * (ny - 1) * (nz - 1)
    hbm, peak_kind = peaks()
    emit_ms = prof.get("slice_emit", (0, 0.0))[1] / args.steps
    algo = 57 * t + 2 * 3 * t * 2 * 4   # outputs (36 + 9 + 12 B per triangle) + the two corner values per vertex
    return {
        "metric": "Mcells/s", "value": round(cells * world / (ms * 1e-3) / 1e6, 1), "unit": "Mcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded fBm generated on the device)",
        "config": {"workload": w["desc"], "volume": [nx, ny, nz], "triangles": int(t),
                   "cache": "volume larger than L2 (4 GiB); each step re-reads only the cut cells' corners"},
        "mtris_per_s": round(t * world / (ms * 1e-3) / 1e6, 1),
        "roofline": {"kernel": "slice_emit", "bound": "hbm", "achieved": round(algo / max(emit_ms, 1e-6) / 1e6, 1),
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(algo / max(emit_ms, 1e-6) / 1e6 / hbm, 4), "algorithmic_bytes_per_launch": int(algo),
                     "launch_ms": round(emit_ms, 4), "traffic": None,
                     "note": "uncut tiles are skipped by a conservative plane bound; the emit is latency-bound "
                             "gathers of the cut cells' corners"},
        "kernels": {kk: {"launches": vv[0], "ms": round(vv[1], 3)} for kk, vv in prof.items()},
        "e2e": None, "gpu_launches": int(launches // max(1, args.steps)), "clocks": clk,
    }


def run_ingest(args, rank, world, local):
    """kvsmc_volume_load_kvsml of a 512^3 float32 external-binary KVSML file."""
    import shutil
    import tempfile
    import time

    import torch

    from kvs_gb300 import _abi
    from kvs_gb300 import ingest

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    nz, ny, nx = w["shape"]
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    d = tempfile.mkdtemp(dir=base)
    try:
        field = make_field(dict(w, kind="fbm"), "cuda").cpu().numpy()
        field.astype("<f4").tofile(os.path.join(d, "vol_value.dat"))
        with open(os.path.join(d, "vol.kvsml"), "w") as f:
            f.write('<?xml version="1.0" ?>\n<KVSML>\n<Object type="StructuredVolumeObject">\n'
                    f'<StructuredVolumeObject grid_type="uniform" resolution="{nx} {ny} {nz}">\n<Node>\n'
                    '<Value veclen="1">\n<DataArray type="float" format="binary" file="vol_value.dat" '
                    'endian="little" />\n</Value>\n</Node>\n</StructuredVolumeObject>\n</Object>\n</KVSML>\n')
        path = os.path.join(d, "vol.kvsml")
        nbytes = field.nbytes
        del field
        for _ in range(args.warmup):
            v, _info = ingest.load_kvsml(ctx, path)
            v.free()
        launches0 = ctx.kernel_launches
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            v, info = ingest.load_kvsml(ctx, path)
            times.append(time.perf_counter() - t0)
            v.free()
        launches = ctx.kernel_launches - launches0
        t = sorted(times)[len(times) // 2]
        gbs = nbytes / t / 1e9
        cpu = None
        if rank == 0 and not args.no_cpu:
            t0 = time.perf_counter()
            reps = 0
            while time.perf_counter() - t0 < 3.0 or reps < 1:
                np.fromfile(os.path.join(d, "vol_value.dat"), "<f4")
                reps += 1
            tc = (time.perf_counter() - t0) / reps
            cpu = {"value": round(nbytes / tc / 1e9, 2), "unit": "GB/s", "cores": 1, "kind": "port",
                   "sample": "the same 512 MiB value file read into host memory (numpy.fromfile: the fread of "
                             "DataArray::ReadExternalData, DataArray.h:175-190), %.1f s on 1 host core" % (tc * reps)}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {
        "metric": "GB/s", "value": round(gbs, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm written as KVSML)",
        "config": {"workload": w["desc"], "bytes": int(nbytes), "timing": "host clock, median of steps"},
        "roofline": {"kernel": "host-to-device link", "bound": "link", "achieved": round(gbs, 2), "peak": None,
                     "unit": "GB/s", "frac": None, "traffic": None,
                     "note": "file (page cache) -> pinned -> HBM; no kernel dominates"},
        "e2e": {"value": round(gbs, 2), "unit": "GB/s", "h2d_bytes_per_step": int(nbytes), "d2h_bytes_per_step": 16,
                "api": "kvsmc_volume_load_kvsml"},
        "gpu_launches": int(launches // max(1, args.steps)), "cpu_baseline": cpu,
    }


def run_stl(args, rank, world, local):
    """kvsmc_stl_records over the device meshes of a multi-isovalue sweep."""
    import time

    import torch

    from kvs_gb300 import _abi
    from kvs_gb300.export import stl_records_device, write_stl_device

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    field = make_field(dict(w, kind="fbm"), "cuda")
    torch.cuda.synchronize()
    vol = _abi.DeviceVolume.from_device(ctx, field.data_ptr(), np.float32, field.shape)
    del field
    torch.cuda.empty_cache()
    n = len(w["isos"])
    reqs = (_abi.Request * n)()
    for i, iso in enumerate(w["isos"]):
        reqs[i].volume = vol.handle
        reqs[i].params = _abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL)
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count")
    meshes = []
    for i in range(n):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        meshes.append((c, nn, s.ntriangles))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
    ctx.check(ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, n), "extract")
    ntri = sum(m[2] for m in meshes)
    offs = np.cumsum([0] + [50 * m[2] for m in meshes])
    out = torch.empty(int(offs[-1]) + 16 * n, dtype=torch.uint8, device="cuda")
    base = out.data_ptr()
    dst = [base + ((int(o) + 15) // 16) * 16 + 16 * i for i, o in enumerate(offs[:-1])]   # 16-byte aligned

    def step():
        for (c, nn, t), d in zip(meshes, dst):
            stl_records_device(ctx, _abi.MODE_DUP_POLYGON_NORMAL, c.data_ptr(), nn.data_ptr(), None, 3 * t, t, d)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ctx.profile_enable(True)
    launches0 = ctx.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = barrier_max(e0.elapsed_time(e1), world) / args.steps
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    hbm, peak_kind = peaks()
    algo = 98 * ntri                      # 48 B of coords + normals read, 50 B of records written
    k_launches, k_ms = prof.get("stl_records", (0, 0.0))
    k_ms_step = k_ms / args.steps
    achieved = algo / (k_ms_step * 1e-3) / 1e9
    e2e = None
    if not args.no_e2e:
        steps = max(1, min(args.steps, 3))
        write_stl_device(ctx, "/dev/null", 0, meshes[0][0].data_ptr(), meshes[0][1].data_ptr(), None,
                         3 * meshes[0][2], meshes[0][2])
        t0 = time.perf_counter()
        for _ in range(steps):
            for c, nn, t in meshes:
                write_stl_device(ctx, "/dev/null", 0, c.data_ptr(), nn.data_ptr(), None, 3 * t, t)
        t_e2e = (time.perf_counter() - t0) / steps
        e2e = {"value": round(ntri / t_e2e / 1e6, 1), "unit": "Mtris/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": int(50 * ntri + 84 * n), "api": "kvsmc_write_stl x%d (to /dev/null)" % n,
               "ms_per_step": round(t_e2e * 1e3, 2)}
    return {
        "metric": "Mtris/s", "value": round(ntri * world / (ms * 1e-3) / 1e6, 1), "unit": "Mtris/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 -> bytes",
        "data": "synthetic (seeded fBm meshes extracted on the device)",
        "config": {"workload": w["desc"], "meshes": n, "triangles": int(ntri),
                   "cache": "inputs larger than L2 (%.1f GB of meshes)" % (48 * ntri / 1e9)},
        "roofline": {"kernel": "stl_records", "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                     "algorithmic_bytes_per_launch": int(algo / max(1, k_launches / args.steps)),
                     "launch_ms": round(k_ms / max(1, k_launches), 4), "traffic": None},
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
        "_sample_mesh": (meshes[0][0][:9 * min(meshes[0][2], 1 << 20)].cpu().numpy(),
                         meshes[0][1][:3 * min(meshes[0][2], 1 << 20)].cpu().numpy()),
    }


def tet_grid(n, seed, device):
    """The tet160 mesh: (values f32[N], coords f32[N, 3], connections int32[C, 4])."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    ar = torch.arange(n, device=device, dtype=torch.float32)
    z, y, x = torch.meshgrid(ar, ar, ar, indexing="ij")
    xyz = torch.stack([x, y, z], -1).reshape(-1, 3)
    xyz = xyz + (torch.rand(xyz.shape, generator=g, device=device) * 0.4 - 0.2)
    c = torch.tensor([80.3, 79.6, 80.9], device=device)
    vals = (torch.sqrt(((xyz - c) ** 2).sum(-1)) + 1.5 * torch.sin(xyz[:, 0] / 7) * torch.sin(xyz[:, 1] / 9)
            * torch.sin(xyz[:, 2] / 11)).float().contiguous()
    m = n - 1
    ai = torch.arange(m, device=device, dtype=torch.int64)
    cz, cy, cx = torch.meshgrid(ai, ai, ai, indexing="ij")
    base = (cx + n * (cy + n * cz)).reshape(-1, 1)
    off = torch.tensor([0, 1, 1 + n, n, n * n, n * n + 1, n * n + 1 + n, n * n + n], device=device)
    hexa = base + off
    del base
    tets = torch.tensor([(0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)],
                        device=device)
    conn = hexa[:, tets].reshape(-1, 4).to(torch.int32).contiguous()
    return vals, xyz.contiguous(), conn


def cells_traffic():
    """DRAM bytes of one tet160 extraction step from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "cells_tet160.json")
    if os.path.exists(p):
        return json.load(open(p)).get("dram_bytes_per_step")
    return None


def run_cells(args, rank, world, local):
    """kvsmc_marching_cells_device on a resident tetrahedral mesh (value), and
    the mapper's host call kvsmc_marching_cells_host from pinned host arrays
    (e2e)."""
    import ctypes as C

    import torch

    from kvs_gb300 import _abi

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    vals, xyz, conn = tet_grid(w["n"], w["seed"] + rank, "cuda")
    nnodes, ncells = vals.numel(), conn.shape[0]
    lo, hi = float(vals.min()), float(vals.max())
    torch.cuda.synchronize()
    s = _abi.Sizes()
    fn = ctx.lib.kvsmc_marching_cells_device

    def call(iso, oc, on, cap):
        return fn(ctx.handle, 0, vals.data_ptr(), 8, nnodes, xyz.data_ptr(), conn.data_ptr(), ncells, iso, 1, lo, hi,
                  oc, 9 * cap, on, 3 * cap, C.byref(s))

    cap = 0
    for r in w["radii"]:
        st = call(r, None, None, 0)
        if st not in (_abi.OK, 6):
            ctx.check(st, "marching_cells_device")
        cap = max(cap, s.ntriangles)
    oc = torch.empty(max(1, 9 * cap), dtype=torch.float32, device="cuda")
    on = torch.empty(max(1, 3 * cap), dtype=torch.float32, device="cuda")
    tris = []

    def step(i):
        ctx.check(call(w["radii"][i % len(w["radii"])], oc.data_ptr(), on.data_ptr(), cap), "marching_cells_device")
        tris.append(s.ntriangles)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    tris.clear()
    clocks = Clocks(local)
    clocks.start()
    ctx.profile_enable(True)
    launches0 = ctx.kernel_launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.steps):
        step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = barrier_max(e0.elapsed_time(e1), world) / args.steps
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    hbm, peak_kind = peaks()
    t_avg = sum(tris) / len(tris)
    # algorithmic bytes of one extraction: the connections once, the values and
    # the coordinates once, the outputs (36 + 12 B per triangle)
    algo = ncells * 16 + nnodes * 4 + nnodes * 12 + 48 * t_avg
    count_ms = prof.get("cells_count", (0, 0.0))[1] / args.steps
    emit_ms = prof.get("cells_emit", (0, 0.0))[1] / args.steps
    line = {
        "metric": "Mcells/s", "value": round(ncells * world / (ms * 1e-3) / 1e6, 1), "unit": "Mcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded mesh and field generated on the device)",
        "config": {"workload": w["desc"], "cells": ncells, "nodes": nnodes, "triangles_per_step": int(t_avg),
                   "cache": "inputs larger than L2 (394 MB of connections per step)"},
        "roofline": {"kernel": "cells_count + cells_emit + scan (whole step)", "bound": "hbm",
                     "achieved": round(algo / (ms * 1e-3) / 1e9, 1), "peak": hbm, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": round(algo / (ms * 1e-3) / 1e9 / hbm, 4),
                     "algorithmic_bytes_per_step": int(algo), "count_ms": round(count_ms, 4),
                     "emit_ms": round(emit_ms, 4), "traffic": cells_traffic()},
        "kernels": {kk: {"launches": vv[0], "ms": round(vv[1], 3)} for kk, vv in prof.items()},
        "gpu_launches": int(launches // max(1, args.steps)), "clocks": clk,
    }
    # a 16-isolevel sweep of the same resident mesh in one call
    # (kvsmc_marching_cells_sweep_device) against 16 single calls
    sweep_isos = [10.0 + 5.0 * i for i in range(16)]
    ns = len(sweep_isos)
    scap = []
    for r in sweep_isos:
        st = call(r, None, None, 0)
        if st not in (_abi.OK, 6):
            ctx.check(st, "marching_cells_device")
        scap.append(max(1, s.ntriangles))
    sbuf_c = [torch.empty(9 * c, dtype=torch.float32, device="cuda") for c in scap]
    sbuf_n = [torch.empty(3 * c, dtype=torch.float32, device="cuda") for c in scap]
    pc = (C.c_void_p * ns)(*[t.data_ptr() for t in sbuf_c])
    pn = (C.c_void_p * ns)(*[t.data_ptr() for t in sbuf_n])
    cc = (C.c_uint64 * ns)(*[9 * c for c in scap])
    cn = (C.c_uint64 * ns)(*[3 * c for c in scap])
    ssz = (_abi.Sizes * ns)()
    il = (C.c_double * ns)(*sweep_isos)

    def sweep():
        ctx.check(ctx.lib.kvsmc_marching_cells_sweep_device(ctx.handle, 0, vals.data_ptr(), 8, nnodes, xyz.data_ptr(),
                                                            conn.data_ptr(), ncells, il, ns, 1, lo, hi, pc, cc, pn,
                                                            cn, ssz), "marching_cells_sweep_device")

    def singles():
        for i, r in enumerate(sweep_isos):
            ctx.check(call(r, sbuf_c[i].data_ptr(), sbuf_n[i].data_ptr(), scap[i]), "marching_cells_device")

    for run in (sweep, singles):
        for _ in range(args.warmup):
            run()
    torch.cuda.synchronize()
    sweep_ms = {}
    for name, run in (("sweep", sweep), ("singles", singles)):
        e0.record(stream)
        for _ in range(max(3, args.steps // 5)):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        sweep_ms[name] = barrier_max(e0.elapsed_time(e1), world) / max(3, args.steps // 5)
    line["sweep16"] = {"call": "kvsmc_marching_cells_sweep_device, 16 isolevels 10..85 in one call",
                       "ms": round(sweep_ms["sweep"], 4),
                       "mcells_isolevels_per_s": round(ncells * ns / (sweep_ms["sweep"] * 1e-3) / 1e6, 1),
                       "triangles": int(sum(x.ntriangles for x in ssz)),
                       "singles_ms": round(sweep_ms["singles"], 4),
                       "speedup_vs_singles": round(sweep_ms["singles"] / sweep_ms["sweep"], 2)}
    del sbuf_c, sbuf_n
    if not args.no_e2e:
        # kvs::SlicePlane on the same mesh (kvsmc_slice_cells_host, the
        # kvs::cuda::SlicePlane call): kernel times from the library's events,
        # and the whole call from pinned host arrays
        from kvs_gb300.marching_cubes import TransferFunction
        from kvs_gb300.slice_plane import slice_cells_host
        hv0, hx0, hk0 = vals.cpu().numpy(), xyz.cpu().numpy(), conn.cpu().numpy().view(np.uint32)
        sp = _abi.SliceParams()
        for i, cf in enumerate((0.31, -0.52, 0.79, -0.31 * 80 + 0.52 * 80 - 0.79 * 80)):
            sp.coefficients[i] = float(np.float32(cf))
        table = np.ascontiguousarray(TransferFunction(256).table, np.uint8)
        sp.tf_min, sp.tf_max, sp.tf_resolution, sp.tf_table = lo, hi, 256, table.ctypes.data
        for _ in range(2):
            slice_cells_host(ctx, 0, hv0, hx0, hk0, sp)
        ctx.profile_enable(True)
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            _, _, _, stri = slice_cells_host(ctx, 0, hv0, hx0, hk0, sp)
        s_ms = (time.perf_counter() - t0) * 1e3 / reps
        sprof = ctx.profile_read()
        ctx.profile_enable(False)
        line["slice"] = {"call": "kvsmc_slice_cells_host, oblique plane (0.31, -0.52, 0.79) through the centre",
                         "triangles": int(stri), "e2e_ms": round(s_ms, 3),
                         "count_ms": round(sprof.get("cells_slice_count", (0, 0.0))[1] / reps, 4),
                         "emit_ms": round(sprof.get("cells_slice_emit", (0, 0.0))[1] / reps, 4)}
        del hv0, hx0, hk0
        hv = torch.empty(vals.shape, dtype=vals.dtype, pin_memory=True)
        hx = torch.empty(xyz.shape, dtype=xyz.dtype, pin_memory=True)
        hk = torch.empty(conn.shape, dtype=conn.dtype, pin_memory=True)
        hv.copy_(vals)
        hx.copy_(xyz)
        hk.copy_(conn)
        del vals, xyz, conn, oc, on
        torch.cuda.empty_cache()
        nv, nx, nk = hv.numpy(), hx.numpy(), hk.numpy().view(np.uint32)
        e2e_tris = []

        def e2e_step(i):
            c, n, sz = _abi.marching_cells_host(ctx, 0, nv, nx, nk, w["radii"][i % len(w["radii"])], (lo, hi))
            e2e_tris.append(sz["ntriangles"])

        for i in range(args.warmup):
            e2e_step(i)
        e2e_tris.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            e2e_step(i)
        torch.cuda.synchronize()
        e_ms = barrier_max((time.perf_counter() - t0) * 1e3, world) / args.steps
        line["e2e"] = {"value": round(ncells * world / (e_ms * 1e-3) / 1e6, 1), "unit": "Mcells/s",
                       "ms_per_step": round(e_ms, 3),
                       "h2d_bytes_per_step": int(nv.nbytes + nx.nbytes + nk.nbytes),
                       "d2h_bytes_per_step": int(48 * sum(e2e_tris) / len(e2e_tris)),
                       "path": "kvsmc_marching_cells_host (the kvs::cuda::MarchingTetrahedra call) from pinned "
                               "host arrays: upload, count, emit, copy back"}
    return line


def cells_cpu_sample(w, planes):
    """A z-slab of the tet160 mesh (full x/y extent, `planes` node planes),
    generated on the CPU with the same formula."""
    vals, xyz, conn = tet_grid(w["n"], w["seed"], "cpu")
    n = w["n"]
    z0 = (n - planes) // 2                      # through the centre: every isolevel cuts it
    nodes = slice(z0 * n * n, (z0 + planes) * n * n)
    cells_per_plane = (n - 1) * (n - 1) * 6
    cells = slice(z0 * cells_per_plane, (z0 + planes - 1) * cells_per_plane)
    return (vals[nodes].numpy(), xyz[nodes].numpy(), (conn[cells] - z0 * n * n).numpy().view(np.uint32))


def run_cells_cpu(w, reference, min_seconds=10.0):
    """The CPU mapper on a 17-plane slab through the centre (2.5 M tetrahedra), one host core,
    cycling the isolevels for at least `min_seconds`: the reference
    MarchingTetrahedra (oracle/_ref) when built, else the numpy restatement
    (oracle/cells.py); returns (Mcells/s, seconds, sample, kind)."""
    vals, xyz, conn = cells_cpu_sample(w, 17)
    ncells = conn.shape[0]
    lo, hi = float(vals.min()), float(vals.max())
    kind = "port"
    if reference:
        from oracle import ref
        if ref.available():
            kind = "reference"
    t0 = time.perf_counter()
    done = 0
    calls = 0
    t = 0.0
    while calls < len(w["radii"]) or time.perf_counter() - t0 < min_seconds:
        r = w["radii"][calls % len(w["radii"])]
        calls += 1
        if kind == "reference":
            from oracle import ref
            # the mapper constructor alone, timed inside oracle/ref_driver.cpp (the
            # volume object's setup copies are left out)
            t += ref.marching_cells(0, vals, xyz, conn, r, minmax=(lo, hi))["seconds"]
        else:
            from oracle import cells as OC
            t1 = time.perf_counter()
            OC.marching_cells(0, vals, xyz, conn, r, (lo, hi))
            t += time.perf_counter() - t1
        done += ncells
    what = ("the reference kvs::MarchingTetrahedra (oracle/_ref)" if kind == "reference"
            else "oracle/cells.py (numpy restatement of kvs::MarchingTetrahedra)")
    return (done / t / 1e6, t, f"{calls} calls (isolevels 30/50/70/90 in turn) on the central 17-plane slab "
            f"({ncells / 1e6:.2f} M tetrahedra), {what}", kind)


def run_stl_ascii(args, rank, world, local):
    """kvsmc_write_stl_ascii of every mesh of a multi-isovalue sweep (text
    formatted on the GPU, copied to pinned memory, written to /dev/null)."""
    import torch

    from kvs_gb300 import _abi
    from kvs_gb300.export import write_stl_ascii_device

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    field = make_field(dict(w, kind="fbm"), "cuda")
    torch.cuda.synchronize()
    vol = _abi.DeviceVolume.from_device(ctx, field.data_ptr(), np.float32, field.shape)
    del field
    torch.cuda.empty_cache()
    n = len(w["isos"])
    reqs = (_abi.Request * n)()
    for i, iso in enumerate(w["isos"]):
        reqs[i].volume = vol.handle
        reqs[i].params = _abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL)
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count")
    meshes = []
    for i in range(n):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        meshes.append((c, nn, s.ntriangles))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
    ctx.check(ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, n), "extract")
    ntri = sum(m[2] for m in meshes)

    def step():
        for c, nn, t in meshes:
            write_stl_ascii_device(ctx, "/dev/null", _abi.MODE_DUP_POLYGON_NORMAL, c.data_ptr(), nn.data_ptr(),
                                   None, 3 * t, t)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ctx.profile_enable(True)
    launches0 = ctx.kernel_launches
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / args.steps
    t = barrier_max(t * 1e3, world) / 1e3
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    # text bytes of one step: the file sizes the writer produced
    import tempfile
    text = 0
    with tempfile.NamedTemporaryFile(suffix=".stl") as f:
        write_stl_ascii_device(ctx, f.name, 0, meshes[0][0].data_ptr(), meshes[0][1].data_ptr(), None,
                               3 * meshes[0][2], meshes[0][2])
        per_tri = os.path.getsize(f.name) / max(1, meshes[0][2])
    text = per_tri * ntri
    hbm, peak_kind = peaks()
    w_launches, w_ms = prof.get("stl_ascii_write", (0, 0.0))
    l_launches, l_ms = prof.get("stl_ascii_len", (0, 0.0))
    k_ms = (w_ms + l_ms) / args.steps
    algo = 48 * ntri + text               # coords + normals read once, the text written once
    achieved = algo / (k_ms * 1e-3) / 1e9 if k_ms else 0.0
    return {
        "metric": "Mtris/s", "value": round(ntri * world / t / 1e6, 1), "unit": "Mtris/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 -> text",
        "data": "synthetic (seeded fBm meshes extracted on the device)",
        "config": {"workload": w["desc"], "meshes": n, "triangles": int(ntri),
                   "text_bytes_per_step": int(text), "timing": "host clock around the whole calls"},
        "gpu_format": {"ms_per_step": round(k_ms, 3), "mtris_per_s": round(ntri / (k_ms * 1e-3) / 1e6, 1)
                       if k_ms else None, "note": "length + write kernels only (CUDA events)"},
        "roofline": {"kernel": "stl_ascii_len + stl_ascii_write", "bound": "hbm", "achieved": round(achieved, 1),
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                     "algorithmic_bytes_per_step": int(algo), "traffic": None},
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "e2e": {"value": round(ntri * world / t / 1e6, 1), "unit": "Mtris/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(text), "api": "kvsmc_write_stl_ascii x%d (to /dev/null)" % n},
        "gpu_launches": int(launches), "clocks": clk,
        "_sample_mesh": (meshes[0][0][:9 * min(meshes[0][2], 20000)].cpu().numpy(),
                         meshes[0][1][:3 * min(meshes[0][2], 20000)].cpu().numpy()),
    }


def run_stl_ascii_cpu(mesh):
    """The ASCII STL restatement (oracle/export.py, the C library's %f through
    Python's formatting) on one host core, on a 20 k-triangle sample."""
    from oracle import export as E
    coords, normals = mesh
    t0 = time.perf_counter()
    E.stl_ascii(coords, normals, np.zeros(0, np.uint32), E.POLYGON_NORMAL)
    t = time.perf_counter() - t0
    return normals.size // 3 / t / 1e6, t, normals.size // 3


def run_stl_cpu(mesh):
    """The STL restatement (oracle/export.py) on one host core, on a 1 M-triangle sample."""
    import time

    from oracle import export as E
    coords, normals = mesh
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < 3.0 or reps < 1:
        E.stl_binary(coords, normals, np.zeros(0, np.uint32), E.POLYGON_NORMAL)
        reps += 1
    t = (time.perf_counter() - t0) / reps
    return normals.size // 3 / t / 1e6, t * reps, normals.size // 3


def run_ours(args, rank, world, local):
    import ctypes as C

    import torch

    from kvs_gb300 import _abi

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    nz, ny, nx = w["shape"]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    tuning = maybe_tune(args, ctx)
    from kvs_gb300 import synthetic as S
    dt = np.dtype(w.get("dtype", np.float32))
    field = make_field(w, "cuda")
    torch.cuda.synchronize()
    vol = _abi.DeviceVolume.from_device(ctx, field.data_ptr(), dt, field.shape)
    host_field = None
    if not args.no_e2e:
        # pinned host buffers next to the GPU's host link
        args.numa = bind_near_gpu(local)
        host_field = torch.empty(field.shape, dtype=field.dtype, pin_memory=True)
        host_field.copy_(field)
    # the CPU baseline's sample: the first z-slab of this same field
    args.cpu_slab = S.to_numpy(field[:min(nz, 65)]) if rank == 0 else None
    sample = None
    if "pcts" in w:
        g = torch.Generator(device="cuda").manual_seed(7)
        src = field.to(torch.int32) if field.dtype == torch.uint16 else field
        sample = src.flatten()[torch.randint(0, field.numel(), (1 << 22,), device="cuda", generator=g)].double()
        sample = sample.cpu().numpy()
        del src
    del field
    torch.cuda.empty_cache()
    isos = workload_isos(w, sample)
    args.isos = isos
    n = len(isos)
    reqs = (_abi.Request * n)()
    mode = w.get("mode", _abi.MODE_DUP_POLYGON_NORMAL)
    args.mode = mode
    for i, iso in enumerate(isos):
        reqs[i].volume = vol.handle
        reqs[i].params = _abi.make_params(iso, mode)
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count")
    outs = []
    for i in range(n):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        k = torch.empty(max(1, s.nconnections), dtype=torch.int32, device="cuda")
        outs.append((c, nn, k))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
        reqs[i].d_connections, reqs[i].connections_capacity = k.data_ptr(), s.nconnections
    ntri = sum(reqs[i].sizes.ntriangles for i in range(n))
    nvert = sum(reqs[i].sizes.nvertices for i in range(n))
    cells = (nx - 1) * (ny - 1) * (nz - 1) * n

    def step():
        ctx.check(ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, n), "extract_batch")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ctx.profile_enable(True)
    launches0 = ctx.kernel_launches
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    if world > 1:
        dist.barrier()
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    ms_max = barrier_max(ms, world)
    step_ms = ms_max / args.steps
    value = cells * world / (step_ms * 1e-3) / 1e6
    # roofline of the dominant kernel (the fused emit launch)
    hbm, peak_kind = peaks()
    algo_bytes = nx * ny * nz * dt.itemsize + 48 * ntri
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    emit_launches, emit_ms = prof.get("stream_emit", (0, 0.0))
    roofline = None
    if mode != _abi.MODE_DUP_POLYGON_NORMAL:
        # shared vertices, over the whole step (several kernel families, none
        # dominant on its own): the volume once per launch that reads it,
        # however many isovalues share the launch, + the outputs: VertexNormal
        # 24 B per vertex (coords, normals) + 12 B per triangle (connections),
        # PolygonNormal 12 B per vertex + 24 B per triangle
        readers = ("stream_count", "snode_count", "snode_emit", "snode_emit_multi", "sconnect", "sconnect_multi",
                   "gather_cell_count", "gather_node_count", "gather_node_emit", "gather_connect")
        passes = sum(prof[k][0] for k in readers if k in prof) / args.steps
        outputs = 24 * nvert + 12 * ntri if mode == _abi.MODE_SHARED_VERTEX_NORMAL else 12 * nvert + 24 * ntri
        algo_bytes = int(nx * ny * nz * dt.itemsize * passes + outputs)
        achieved = algo_bytes / (step_ms * 1e-3) / 1e9
        roofline = {"kernel": "whole step (shared-vertex passes)", "bound": "hbm", "achieved": round(achieved, 1),
                    "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                    "algorithmic_bytes_per_step": algo_bytes, "volume_passes_per_step": round(passes, 2),
                    "traffic": None}
    elif emit_launches:
        per = emit_ms / emit_launches
        achieved = algo_bytes / (per * 1e-3) / 1e9
        tr = traffic_per_launch(args.workload)
        roofline = {"kernel": "stream_emit", "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm,
                    "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                    "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": round(per, 4),
                    "traffic": tr}
    # end to end through the C ABI with host buffers
    e2e = None
    if host_field is not None:
        e2e = run_e2e(ctx, host_field, isos, reqs, args, stream, mode)
        if e2e is not None:
            e2e["value"] = round(cells / (e2e.pop("step_ms") * 1e-3) / 1e6 * world, 1)
            e2e["unit"] = "Mcells/s"
    line = {
        "metric": "Mcells/s", "value": round(value, 1), "unit": "Mcells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"float32": "f32", "uint16": "u16"}.get(dt.name, dt.name),
        "data": "synthetic (seeded field generated on the device)",
        "config": {"workload": w["desc"], "volume": [nx, ny, nz], "isovalues": n,
                   "isolevels": [round(x, 6) for x in isos],
                   "mode": {0: "duplication+PolygonNormal", 1: "shared vertices+PolygonNormal",
                            2: "VertexNormal (shared vertices)"}[mode],
                   "cache": "inputs larger than L2 (4 GiB volume, "
                   "outputs ~48 B/triangle)" if args.workload in ("sweep1024", "sweep1024vn", "heavy") else (
                   "inputs larger than L2 (512 MiB volume)" if args.workload == "sweep512" else "input smaller than L2"),
                   "launch_shapes": "autotuned (--tune)" if tuning else "built-in rules"},
        "tuning": tuning,
        "mtris_per_s": round(ntri * world / (step_ms * 1e-3) / 1e6, 1),
        "triangles_per_step": int(ntri),
        "vertices_per_step": int(nvert),
        "roofline": roofline,
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "dominant_kernel": dom[0],
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    # parity of this step's outputs at the bench size, after the timed region
    if not args.no_verify and rank == 0:
        v = (verify_outputs(ctx, vol, w, reqs, outs, isos) if mode == _abi.MODE_DUP_POLYGON_NORMAL
             else verify_shared(vol, reqs, outs, isos))
        line["verified"] = v["verified"]
        line["verify"] = v
    return line


def verify_outputs(ctx, vol, w, reqs, outs, isos, planes=2, chunk_tris=1 << 20):
    """Check the step's device outputs against the C oracle (oracle/mc_oracle.c)
    without copying them back: per isovalue, position-keyed checksums of the
    coords (9 words per triangle) and normals (3 per triangle) arrays in chunks
    of 2^20 triangles (kvsmc_checksum_words on the device, mco_dup_checksum on
    the host) and the triangle count.  Whole volume for the sweep and blob
    workloads (every triangle of every output); for the 8 GiB stress volume
    the first and last `planes` cell planes, compared with the first and last
    triangles of each output (the last planes' node indices pass 2^32).
    Runs after the timed region; isovalues on all host threads."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    host = vol.download()
    nz, ny, nx = host.shape
    cz = nz - 1
    full = w["kind"] != "lattice"
    slabs = [(0, cz)] if full else [(0, planes), (cz - planes, cz)]
    jobs = [(i, z0, z1) for i in range(len(isos)) for (z0, z1) in slabs]

    def run(job):
        i, z0, z1 = job
        p = reqs[i].params
        s = reqs[i].sizes
        return oracle.dup_checksum(host, p.isolevel, s.min_value, s.max_value, z0, z1,
                                   min_coord=tuple(p.min_coord), scale=tuple(p.scale), chunk_tris=chunk_tris)

    with cf.ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        results = dict(zip(jobs, ex.map(run, jobs)))
    t_oracle = time.perf_counter() - t0
    per_iso, ok = [], True
    for i, iso in enumerate(isos):
        T = int(reqs[i].sizes.ntriangles)
        entry = {"isovalue": round(float(iso), 6), "triangles": T, "slabs": []}
        for (z0, z1) in slabs:
            t, cs, ns = results[(i, z0, z1)]
            first = 0 if z0 == 0 else T - t
            sl = {"planes": [z0, z1], "triangles": int(t), "first_triangle": int(first)}
            if full and t != T:
                sl["count_mismatch"] = [int(t), T]
                ok = False
            elif t:
                c, n = outs[i][:2]
                gc = ctx.checksum_words(c.data_ptr() + 4 * 9 * first, 9 * t, 9 * chunk_tris)
                gn = ctx.checksum_words(n.data_ptr() + 4 * 3 * first, 3 * t, 3 * chunk_tris)
                bad = [k for k in range(len(cs)) if cs[k] != gc[k] or ns[k] != gn[k]]
                sl["coords_sum"] = f"{int(cs.sum(dtype=np.uint64)):016x}"
                sl["normals_sum"] = f"{int(ns.sum(dtype=np.uint64)):016x}"
                if bad:
                    k = bad[0]
                    sl["first_diff"] = {"chunk": k, "triangles": [first + k * chunk_tris,
                                                                  first + min(t, (k + 1) * chunk_tris)],
                                        "chunks_differing": len(bad)}
                    ok = False
            entry["slabs"].append(sl)
        per_iso.append(entry)
    return {"verified": ok, "oracle": "oracle/mc_oracle.c (mco_dup_checksum), one isovalue per host thread",
            "method": "triangle counts + position-keyed checksums per 2^20 triangles of every coords and normals "
                      "word (kvsmc_checksum_words on the device)",
            "scope": "whole volume, every output" if full else
                     f"first and last {planes} cell planes of every output",
            "seconds": round(time.perf_counter() - t0, 1), "oracle_seconds": round(t_oracle, 1),
            "isolevels": per_iso}


def verify_shared(vol, reqs, outs, isos, max_checked=2):
    """Shared-vertex outputs against the oracle's whole arrays (coords,
    connections, normals), bit for bit, for the middle isovalue(s): the
    oracle's vertex map costs 12 B per node, so a 1024^3 volume takes one
    isovalue at a time.  Runs after the timed region."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    host = vol.download()
    n = len(isos)
    picks = sorted({n // 2, max(0, n // 2 - 1)})[:max_checked] if n > 1 else [0]
    per, ok = [], True
    for i in picks:
        p, s = reqs[i].params, reqs[i].sizes
        o = oracle.extract(host, p.isolevel, p.mode, s.min_value, s.max_value, tuple(p.min_coord), tuple(p.scale))
        c, nn, k = outs[i]
        e = {"isovalue": round(float(isos[i]), 6), "triangles": int(s.ntriangles), "vertices": int(s.nvertices)}
        for name, got, ref in (("coords", c[:s.ncoords], o["coords"]), ("normals", nn[:s.nnormals], o["normals"]),
                               ("connections", k[:s.nconnections], o["connections"])):
            g = got.cpu().numpy()
            g = g.view(np.uint32) if name == "connections" else g
            r = ref.view(np.uint32) if name != "connections" else ref
            same = g.size == ref.size and np.array_equal(g.view(np.uint32), r.view(np.uint32))
            if not same:
                ok = False
                d = np.nonzero(g.view(np.uint32)[:min(g.size, r.size)] != r.view(np.uint32)[:min(g.size, r.size)])[0]
                e[name + "_first_diff"] = int(d[0]) if d.size else [int(g.size), int(ref.size)]
        per.append(e)
        del o
    return {"verified": ok, "oracle": "oracle/mc_oracle.c (mco_extract, whole arrays)",
            "method": "bit-exact comparison of coords, connections and vertex normals",
            "scope": f"isovalues {[round(float(isos[i]), 4) for i in picks]} of {n}, whole volume",
            "seconds": round(time.perf_counter() - t0, 1), "isolevels": per}


def gpu_numa_node(local):
    """NUMA node of the GPU's PCI function (sysfs), or None."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(local)
        bdf = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        n = int(open(f"/sys/bus/pci/devices/{bdf}/numa_node").read().strip())
        return n if n >= 0 else None
    except Exception:
        return None


def node_cpus(node):
    """CPUs of a NUMA node (sysfs cpulist), or an empty set."""
    try:
        text = open(f"/sys/devices/system/node/node{node}/cpulist").read().strip()
    except OSError:
        return set()
    out = set()
    for part in text.split(","):
        if "-" in part:
            a, b = part.split("-")
            out.update(range(int(a), int(b) + 1))
        elif part:
            out.add(int(part))
    return out


def bind_near_gpu(local):
    """Run this process on the host CPUs of the GPU's NUMA node (where they are
    among the allowed ones), so pinned buffers allocated afterwards sit next to
    the GPU's host link.  Returns what was done."""
    node = gpu_numa_node(local)
    info = {"gpu_numa_node": node}
    if node is None or not hasattr(os, "sched_setaffinity"):
        return info
    allowed = os.sched_getaffinity(0)
    near = node_cpus(node) & allowed
    if near and near != allowed:
        os.sched_setaffinity(0, near)
        info["bound_cpus"] = len(near)
    return info


def page_numa_node(addr):
    """NUMA node holding the page at a host address (move_pages query), or None."""
    import ctypes
    import platform
    nr = {"x86_64": 279, "aarch64": 239}.get(platform.machine())
    if nr is None:
        return None
    try:
        libc = ctypes.CDLL(None, use_errno=True)
        pages = (ctypes.c_void_p * 1)(addr & ~4095)
        status = (ctypes.c_int * 1)(-1)
        r = libc.syscall(ctypes.c_long(nr), ctypes.c_int(0), ctypes.c_ulong(1), pages, None, status,
                         ctypes.c_int(0))
        return int(status[0]) if r == 0 and status[0] >= 0 else None
    except Exception:
        return None


def run_e2e(ctx, host_field, isos, reqs, args, stream, mode=0):
    """Same sweep through kvsmc_extract_batch_host: H2D of the volume from
    pinned memory, the passes, D2H of every output into pinned buffers."""
    import torch

    from kvs_gb300 import _abi
    n = len(isos)
    pinned = {}
    for i in range(n):
        s = reqs[i].sizes
        pinned[(i, 0)] = torch.empty(max(1, s.ncoords), dtype=torch.float32, pin_memory=True).numpy()
        pinned[(i, 1)] = torch.empty(max(1, s.nnormals), dtype=torch.float32, pin_memory=True).numpy()
        if mode != _abi.MODE_DUP_POLYGON_NORMAL:
            pinned[(i, 2)] = torch.empty(max(1, s.nconnections), dtype=torch.int32,
                                         pin_memory=True).numpy().view(np.uint32)
    params = [_abi.make_params(iso, mode) for iso in isos]
    host = host_field.numpy()

    def buf(req, kind, count):
        a = pinned.get((req, kind))
        return a if a is not None and a.size >= count else None

    steps = max(3, min(args.steps, 5))
    for _ in range(2):
        _abi.extract_batch_host(ctx, host, params, buf)
    torch.cuda.synchronize()
    times = []
    ctx.profile_enable(True)
    for _ in range(steps):
        t0 = time.perf_counter()
        out = _abi.extract_batch_host(ctx, host, params, buf)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    t = statistics.median(times)   # the call is host-bound (link transfers): the median damps host noise
    h2d = host.nbytes
    d2h = sum(o["coords"].nbytes + o["normals"].nbytes + o["connections"].nbytes for o in out)
    link = {}
    for name, nbytes in (("copy_h2d", h2d), ("copy_d2h", d2h)):
        n, ms = prof.get(name, (0, 0.0))
        if n and ms > 0:
            # device-side time of the copies (CUDA events on the copy's own stream)
            link[name.replace("copy_", "") + "_GBs"] = round(nbytes * steps / (ms * 1e-3) / 1e9, 1)
    link["pinned_numa_nodes"] = sorted({page_numa_node(host.ctypes.data)} |
                                       {page_numa_node(a.ctypes.data) for a in list(pinned.values())[:4]} - {None})
    link.update(getattr(args, "numa", {}))
    return {"step_ms": t * 1e3, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "api": "kvsmc_extract_batch_host", "steps": steps, "timing": "host clock, median of steps",
            "pipeline": ("emit in 8 launches by plane ranges, each range's triangles copied to the host on a "
                         "second stream while the next range is written") if mode == _abi.MODE_DUP_POLYGON_NORMAL else
                        ("one count, one node emit and one connection pass for all the requests, then each "
                         "request's vertex normals; each request's vertices, connections and normals copied "
                         "to the host on a second stream as soon as the pass that writes them ends"),
            "link": link,
            "kernels_ms_per_step": {k: round(v[1] / steps, 3) for k, v in prof.items()}}


# ----------------------------------------------------------------- uneven batch

def run_batch(args, rank, world, local):
    """The uneven multi-volume batch: plain per-call vs batched vs graph replay."""
    import ctypes as C

    import torch

    from kvs_gb300 import _abi
    from kvs_gb300 import synthetic as S

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    tuning = maybe_tune(args, ctx)
    rng = np.random.default_rng(w["seed"])
    dts = [np.uint8, np.uint16, np.float32]
    vols, params, hosts, shapes = [], [], [], []
    cells = 0
    in_bytes = 0
    sample = []
    for i in range(w["n"]):
        nz, ny, nx = (int(d) for d in rng.integers(w["dims"][0], w["dims"][1] + 1, 3))
        dt = dts[int(rng.integers(0, 3))]
        f = S.ellipsoid_phantom((nz, ny, nx), dt, seed=w["seed"] + 1 + i, device="cuda")
        torch.cuda.synchronize()
        dv = _abi.DeviceVolume.from_device(ctx, f.data_ptr(), dt, (nz, ny, nx))
        if not args.no_e2e:
            h = torch.empty(f.shape, dtype=f.dtype, pin_memory=True)
            h.copy_(f)
            hosts.append(h)
        if rank == 0 and len(sample) < 4:
            sample.append(S.to_numpy(f))
        del f
        mn, mx = dv.minmax()
        iso = mn + rng.uniform(0.2, 0.8) * (mx - mn)
        vols.append(dv)
        params.append(_abi.make_params(iso, _abi.MODE_DUP_POLYGON_NORMAL))
        shapes.append((nz, ny, nx, np.dtype(dt)))
        cells += (nx - 1) * (ny - 1) * (nz - 1)
        in_bytes += nx * ny * nz * np.dtype(dt).itemsize
    torch.cuda.empty_cache()
    n = len(vols)
    reqs = (_abi.Request * n)()
    for i in range(n):
        reqs[i].volume = vols[i].handle
        reqs[i].params = params[i]
    ctx.check(ctx.lib.kvsmc_count_batch(ctx.handle, reqs, n), "count")
    outs = []
    for i in range(n):
        s = reqs[i].sizes
        c = torch.empty(max(1, s.ncoords), dtype=torch.float32, device="cuda")
        nn = torch.empty(max(1, s.nnormals), dtype=torch.float32, device="cuda")
        outs.append((c, nn))
        reqs[i].d_coords, reqs[i].coords_capacity = c.data_ptr(), s.ncoords
        reqs[i].d_normals, reqs[i].normals_capacity = nn.data_ptr(), s.nnormals
    ntri = sum(reqs[i].sizes.ntriangles for i in range(n))
    sizes = _abi.Sizes()

    def per_call():
        for i in range(n):
            ctx.check(ctx.lib.kvsmc_extract_device(ctx.handle, vols[i].handle, C.byref(reqs[i].params),
                                                   reqs[i].d_coords, reqs[i].coords_capacity, reqs[i].d_normals,
                                                   reqs[i].normals_capacity, None, 0, C.byref(sizes)),
                      "extract_device")

    def batched():
        ctx.check(ctx.lib.kvsmc_extract_batch(ctx.handle, reqs, n), "extract_batch")

    plan = _abi.Plan(ctx, reqs)

    def replay():
        plan.launch()
        plan.wait()

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        launches0 = ctx.kernel_launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return barrier_max(e0.elapsed_time(e1), world) / steps, (ctx.kernel_launches - launches0) // steps

    ms_call, l_call = timed(per_call, max(1, args.steps // 2))
    ms_batch, l_batch = timed(batched, args.steps)
    clocks = Clocks(local)
    clocks.start()
    ms_graph, l_graph = timed(replay, args.steps)
    clk = clocks.stop()
    # kernel times of one batch (same kernels as the replay) for the roofline
    ctx.profile_enable(True)
    batched()
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    hbm, peak_kind = peaks()
    algo = in_bytes + 48 * ntri
    emit_ms = sum(v[1] for k, v in prof.items() if k == "stream_emit")
    count_ms = sum(v[1] for k, v in prof.items() if k == "stream_count")
    # the per-kind launches overlap, so the roofline is taken over the whole
    # replayed step (count + scans + emit): algorithmic bytes / step time
    roofline = {"kernel": "whole plan replay", "bound": "hbm", "achieved": round(algo / (ms_graph * 1e-3) / 1e9, 1),
                "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                "frac": round(algo / (ms_graph * 1e-3) / 1e9 / hbm, 4), "algorithmic_bytes_per_launch": int(algo),
                "launch_ms": round(ms_graph, 4), "traffic": None,
                "note": "per-kind count and emit launches run side by side; kernel ms below are summed per family "
                        "(emit %.2f, count %.2f) and overlap" % (emit_ms, count_ms)}
    mc = lambda ms: round(cells * world / (ms * 1e-3) / 1e6, 1)
    e2e = None
    if hosts:
        host_out = [(torch.empty(c.shape, dtype=c.dtype, pin_memory=True),
                     torch.empty(nn.shape, dtype=nn.dtype, pin_memory=True)) for c, nn in outs]

        def e2e_step():
            for i in range(n):
                ctx.check(ctx.lib.kvsmc_volume_update(ctx.handle, vols[i].handle, hosts[i].data_ptr()), "update")
            plan.launch()
            with torch.cuda.stream(stream):
                for (c, nn), (hc, hn) in zip(outs, host_out):
                    hc.copy_(c, non_blocking=True)
                    hn.copy_(nn, non_blocking=True)
            plan.wait()
            stream.synchronize()

        ms_e2e, _ = timed(e2e_step, max(1, args.steps // 2))
        e2e = {"value": mc(ms_e2e), "unit": "Mcells/s", "h2d_bytes_per_step": int(in_bytes),
               "d2h_bytes_per_step": int(sum(4 * (c.numel() + nn.numel()) for c, nn in outs)),
               "api": "kvsmc_volume_update x200 + kvsmc_plan_launch/wait + device-to-host copies", "ms_per_step": round(ms_e2e, 3)}
    plan.close()
    args.batch_sample = sample
    args.batch_params = [(params[i].isolevel, reqs[i].sizes.min_value, reqs[i].sizes.max_value) for i in range(4)]
    return {
        "metric": "Mcells/s", "value": mc(ms_graph), "unit": "Mcells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_graph, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u16/f32", "data": "synthetic (seeded phantoms generated on the device)",
        "config": {"workload": w["desc"], "requests": n, "cells": int(cells), "input_bytes": int(in_bytes),
                   "cache": "inputs larger than L2 (%.1f GB of volumes)" % (in_bytes / 1e9),
                   "launch_shapes": "autotuned (--tune)" if tuning else "built-in rules"},
        "tuning": tuning,
        "mtris_per_s": round(ntri * world / (ms_graph * 1e-3) / 1e6, 1), "triangles_per_step": int(ntri),
        "forms": {"per_call": {"api": "kvsmc_extract_device x%d" % n, "ms_per_step": round(ms_call, 3),
                               "value": mc(ms_call), "gpu_launches": int(l_call)},
                  "batched": {"api": "kvsmc_extract_batch", "ms_per_step": round(ms_batch, 3),
                              "value": mc(ms_batch), "gpu_launches": int(l_batch)},
                  "graph": {"api": "kvsmc_plan_launch + kvsmc_plan_wait", "ms_per_step": round(ms_graph, 3),
                            "value": mc(ms_graph), "gpu_launches": int(l_graph)}},
        "speedup_vs_per_call": round(ms_call / ms_graph, 2),
        "roofline": roofline,
        "kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof.items()},
        "e2e": e2e, "gpu_launches": int(l_graph), "clocks": clk,
    }


def run_batch_cpu(args):
    """The oracle on the first sample volumes of the batch, one core."""
    from oracle import oracle
    oracle.build()
    done, t = 0, 0.0
    for v, (iso, mn, mx) in zip(args.batch_sample, args.batch_params):
        nz, ny, nx = v.shape
        t0 = time.perf_counter()
        oracle.extract(v, iso, 0, mn, mx)
        t += time.perf_counter() - t0
        done += (nx - 1) * (ny - 1) * (nz - 1)
    return done / t / 1e6, t, "%d volumes of the batch (%s), %.0f M cells" % (
        len(args.batch_sample), ", ".join("x".join(str(d) for d in v.shape[::-1]) + " " + str(v.dtype)
                                          for v in args.batch_sample), done / 1e6)


# ----------------------------------------------------------------- serving

def run_serve(args, rank, world, local):
    """The request loop under Poisson arrivals: p50/p99 latency and throughput."""
    import threading

    import torch

    from kvs_gb300 import _abi
    from kvs_gb300 import synthetic as S

    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ctx = _abi.Context(local)
    rng = np.random.default_rng(w["seed"])
    vols, pct, cells = [], [], []
    for i, (kind, shape, dt) in enumerate(w["volumes"]):
        if kind == "fbm":
            f = S.fbm(shape, seed=w["seed"] + i, device="cuda")
        elif kind == "phantom":
            f = S.ellipsoid_phantom(shape, dt, seed=w["seed"] + i, device="cuda")
        else:
            f = S.gaussian_blobs(shape, seed=w["seed"] + i, device="cuda")
        torch.cuda.synchronize()
        vols.append(_abi.DeviceVolume.from_device(ctx, f.data_ptr(), dt, shape))
        g = torch.Generator(device="cuda").manual_seed(i)
        src = f.to(torch.int32) if f.dtype == torch.uint16 else f   # no uint16 indexing on every torch
        sample = src.flatten()[torch.randint(0, f.numel(), (1 << 20,), device="cuda", generator=g)].double()
        pct.append((float(torch.quantile(sample, 0.10)), float(torch.quantile(sample, 0.90))))
        cells.append((shape[0] - 1) * (shape[1] - 1) * (shape[2] - 1))
        del f, src, sample
    torch.cuda.empty_cache()
    for v in vols:
        v.minmax()
    srv = _abi.Server(ctx, budget_bytes=40 << 30, max_batch=256, workers=3)

    def run_rate(rate, seconds, warm=False):
        n = max(20, int(rate * seconds))
        gaps = rng.exponential(1.0 / rate, n)
        picks = rng.integers(0, len(vols), n)
        fr = rng.uniform(0.0, 1.0, n)
        reqs = [(int(picks[k]), _abi.make_params(pct[picks[k]][0] + fr[k] * (pct[picks[k]][1] - pct[picks[k]][0]),
                                                 _abi.MODE_DUP_POLYGON_NORMAL)) for k in range(n)]
        done = []

        def poller():
            t_end = time.time() + 600
            while len(done) < n and time.time() < t_end:
                for c in srv.poll(timeout_ms=50):
                    done.append((c.ticket, c.status, c.submit_s, c.start_s, c.done_s, c.sizes.ntriangles,
                                 c.batch_size))
                    srv.release(c.ticket)

        th = threading.Thread(target=poller)
        th.start()
        vol_of = {}
        t_next = time.perf_counter()
        for k in range(n):
            t_next += gaps[k]
            while True:
                d = t_next - time.perf_counter()
                if d <= 0:
                    break
                if d > 0.0003:
                    time.sleep(d - 0.0002)
            vol_of[srv.submit(vols[reqs[k][0]], reqs[k][1])] = reqs[k][0]
        th.join()
        if warm:
            return None
        lat = np.array([d[4] - d[2] for d in done]) * 1e3
        span = max(d[4] for d in done) - min(d[2] for d in done)
        served = [d for d in done if d[1] == 0]
        tri = sum(d[5] for d in served)
        cel = sum(cells[vol_of[d[0]]] for d in served)
        return {"rate_req_s": rate, "requests": n, "completed": len(done), "ok": len(served),
                "refused_budget": sum(1 for d in done if d[1] == _abi.ERR_BUDGET),
                "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "mean_ms": round(float(lat.mean()), 3),
                "queue_p50_ms": round(float(np.percentile([(d[3] - d[2]) * 1e3 for d in done], 50)), 3),
                "throughput_req_s": round(len(served) / span, 1), "mcells_per_s": round(cel / span / 1e6, 1),
                "gb_written_per_s": round(48 * tri / span / 1e9, 1),
                "mtris_per_s": round(tri / span / 1e6, 1),
                "mean_batch": round(float(np.mean([d[6] for d in done])), 2)}

    run_rate(200, 0.5, warm=True)
    clocks = Clocks(local)
    clocks.start()
    launches0 = srv.stats()["kernel_launches"]
    results = [run_rate(r, w["seconds"]) for r in w["rates"]]
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    top = results[-1]
    return {
        "metric": "Mcells/s", "value": top["mcells_per_s"], "unit": "Mcells/s", "n_gpus": world,
        "steps": len(results), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16/f32", "data": "synthetic (seeded fields generated on the device)",
        "config": {"workload": w["desc"], "budget_bytes": 40 << 30, "max_batch": 256, "workers": 3,
                   "cache": "volumes 4.2 GB in all, larger than L2"},
        "value_at": "%d req/s offered (served requests only; a result larger than the budget alone is refused "
                    "with KVSMC_ERR_BUDGET)" % top["rate_req_s"],
        "serving": results,
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
        "server_stats": st, "gpu_launches": int(st["kernel_launches"] - launches0), "clocks": clk,
        "e2e": None,
    }


# ----------------------------------------------------------------- CPU side

def cpu_slab_sample(args, slab_planes):
    """A z-slab of the workload's field (generated on the CPU, same generator)."""
    import torch
    from kvs_gb300 import synthetic as S
    w = WORKLOADS[args.workload]
    nz, ny, nx = w["shape"]
    if w["kind"] == "fbm":
        # same field: generate the full-depth statistics on a slab (rescaled
        # per slab; the sample only sets the cost per cell)
        f = S.fbm((slab_planes, ny, nx), seed=42, device="cpu")
    elif w["kind"] == "lattice":
        # lattice noise is statistically the same in every slab
        f = S.lattice_noise((min(slab_planes, nz), ny, nx), w["dtype"], seed=42, device="cpu", spacing=w["spacing"])
    else:
        f = S.gaussian_blobs((min(slab_planes, nz), ny, nx), seed=42, device="cpu")
    return S.to_numpy(f)


def run_cpu(args, threads, planes, isos):
    """The oracle (C restatement of kvs::MarchingCubes) over (isovalue) units on
    `threads` host threads; returns (cells x isovalues)/s and the sample text."""
    from oracle import oracle
    oracle.build()
    v = getattr(args, "cpu_slab", None)
    if v is None:
        v = cpu_slab_sample(args, planes)
    vmin, vmax = float(v.min()), float(v.max())
    nz, ny, nx = v.shape
    cells = (nx - 1) * (ny - 1) * (nz - 1)

    mode = getattr(args, "mode", 0)

    def one(iso):
        oracle.extract(v, iso, mode, vmin, vmax)
        return cells

    t0 = time.perf_counter()
    if threads == 1:
        done = sum(one(i) for i in isos)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            done = sum(ex.map(one, isos))
    t = time.perf_counter() - t0
    mode_name = {0: "duplication+PolygonNormal", 1: "shared vertices+PolygonNormal", 2: "VertexNormal"}[mode]
    return (done / t / 1e6, t,
            f"{len(isos)} isovalues x {nx}x{ny}x{nz} slab ({done / 1e6:.0f} M cell-isovalues, {mode_name})")


def batch_reference_sample(w, count):
    """The first `count` requests of a batch workload, generated on the CPU
    with the same generator, shapes, dtypes and isovalues as the GPU run."""
    from kvs_gb300 import synthetic as S
    rng = np.random.default_rng(w["seed"])
    dts = [np.uint8, np.uint16, np.float32]
    out = []
    for i in range(count):
        nz, ny, nx = (int(d) for d in rng.integers(w["dims"][0], w["dims"][1] + 1, 3))
        dt = dts[int(rng.integers(0, 3))]
        v = S.to_numpy(S.ellipsoid_phantom((nz, ny, nx), dt, seed=w["seed"] + 1 + i, device="cpu"))
        mn, mx = float(v.min()), float(v.max())
        iso = mn + rng.uniform(0.2, 0.8) * (mx - mn)
        out.append((v, iso, mn, mx))
    return out


def run_reference_batch(args, world, threads):
    from oracle import oracle
    oracle.build()
    w = WORKLOADS[args.workload]
    reqs = batch_reference_sample(w, 12)
    cells = sum((v.shape[0] - 1) * (v.shape[1] - 1) * (v.shape[2] - 1) for v, _, _, _ in reqs)

    def one(r):
        v, iso, mn, mx = r
        oracle.extract(v, iso, 0, mn, mx)

    vals = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(one, reqs))
        t = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(t)
    t = statistics.median(vals)
    value = cells / t / 1e6
    sample = f"first {len(reqs)} requests of the batch ({cells / 1e6:.0f} M cells), one request per thread"
    return {
        "impl": "reference", "metric": "Mcells/s", "value": round(value, 1), "unit": "Mcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16/f32", "data": "synthetic",
        "config": {"workload": w["desc"], "sample": sample},
        "cpu_baseline": {"value": round(value, 1), "unit": "Mcells/s", "cores": min(threads, len(reqs)),
                         "kind": "port",
                         "sample": sample + "; oracle/mc_oracle.c (C restatement of kvs::MarchingCubes, "
                         "-O3 -ffp-contract=off)"},
        "e2e": {"value": round(value, 1), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def reference_line(args, world, w, metric, value, ms, sample, dtype="f32"):
    """The reference arm's JSON line for a workload timed on one host core."""
    return {
        "impl": "reference", "metric": metric, "value": round(value, 3), "unit": metric, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
        "config": {"workload": w["desc"], "sample": sample},
        "cpu_baseline": {"value": round(value, 3), "unit": metric, "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": metric, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference_stl(args, world, w):
    """kvs::Stl's writer (binary, or the ASCII default) restated in
    oracle/export.py, on one host core, over meshes of the workload's field:
    the workload's isovalues on a 65-plane slab, extracted by the oracle."""
    from oracle import oracle
    oracle.build()
    v = cpu_slab_sample(args, 65)
    outs = [oracle.extract(v, iso, 0, float(v.min()), float(v.max())) for iso in w["isos"]]
    ascii_ = w["kind"] == "stlascii"
    coords = np.concatenate([o["coords"] for o in outs])
    normals = np.concatenate([o["normals"] for o in outs])
    nt = min(normals.size // 3, 20000 if ascii_ else 1 << 20)
    mesh = (coords[:9 * nt], normals[:3 * nt])
    vals = []
    for i in range(args.warmup + args.steps):
        mt, t, _ = (run_stl_ascii_cpu if ascii_ else run_stl_cpu)(mesh)
        if i >= args.warmup:
            vals.append((mt, nt / mt / 1e3))
    value = statistics.median(x for x, _ in vals)
    ms = statistics.median(x for _, x in vals)
    sample = (f"{nt} triangles of the {len(w['isos'])} isovalues' meshes of a 65-plane slab of the field, "
              f"{'ASCII' if ascii_ else 'binary'} STL records; oracle/export.py (restatement of kvs::Stl's writer)")
    return reference_line(args, world, w, "Mtris/s", value, ms, sample, "f32 -> bytes")


def run_reference_slice(args, world, w):
    """kvs::SlicePlane's extract_plane restated in oracle/slice.py (every cell
    visited, as the reference does) on one host core, over a z-slab of the
    workload's field cut by the workload's plane normal through the slab's
    centre."""
    from kvs_gb300.marching_cubes import TransferFunction
    from oracle import slice as OS
    nz, ny, nx = w["shape"]
    planes = max(2, min(nz, (1 << 24) // (nx * ny) + 1))
    v = cpu_slab_sample(args, planes)
    f32 = np.float32
    pt = np.array([w["point"][0], w["point"][1], (planes - 1) / 2], f32)
    nrm = np.array(w["normal"], f32)
    dot = f32(f32(f32(pt[0] * nrm[0]) + f32(pt[1] * nrm[1])) + f32(pt[2] * nrm[2]))
    coef = np.array([nrm[0], nrm[1], nrm[2], -dot], f32)
    table = TransferFunction(256).table
    lo, hi = f32(v.min()), f32(v.max())
    cells = (nx - 1) * (ny - 1) * (planes - 1)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        OS.slice_plane(v, coef, table, lo, hi)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    sample = (f"{nx}x{ny}x{planes} slab of the field ({cells / 1e6:.0f} M cells), the workload's plane normal through "
              f"the slab's centre; oracle/slice.py (restatement of SlicePlane::extract_plane)")
    return reference_line(args, world, w, "Mcells/s", cells / t / 1e6, t * 1e3, sample)


def run_reference_ingest(args, world, w):
    """The reference's external-binary KVSML read (the fread of
    DataArray::ReadExternalData, DataArray.h:175-190) as numpy.fromfile on one
    host core, over a 128 MiB float32 value file in the page cache."""
    import shutil
    import tempfile
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    d = tempfile.mkdtemp(dir=base)
    try:
        path = os.path.join(d, "vol_value.dat")
        nbytes = 128 << 20
        np.random.default_rng(1).random(nbytes // 4, dtype=np.float32).astype("<f4").tofile(path)
        times = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            np.fromfile(path, "<f4")
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    t = statistics.median(times)
    sample = "a 128 MiB float32 value file in the page cache read into host memory (numpy.fromfile)"
    return reference_line(args, world, w, "GB/s", nbytes / t / 1e9, t * 1e3, sample)


def run_reference(args, rank, world):
    if rank != 0:
        return None
    w = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    if w["kind"] == "batch":
        return run_reference_batch(args, world, threads)
    if w["kind"] in ("stl", "stlascii"):
        return run_reference_stl(args, world, w)
    if w["kind"] == "slice":
        return run_reference_slice(args, world, w)
    if w["kind"] == "ingest":
        return run_reference_ingest(args, world, w)
    if w["kind"] == "cells":
        vals = []
        for i in range(args.warmup + args.steps):
            v, t, sample, kind = run_cells_cpu(w, reference=True, min_seconds=3.0)
            if i >= args.warmup:
                vals.append((v, t))
        value = statistics.median(v for v, _ in vals)
        ms = statistics.median(t for _, t in vals) * 1e3
        return {
            "impl": "reference", "metric": "Mcells/s", "value": round(value, 1), "unit": "Mcells/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "sample": sample},
            "cpu_baseline": {"value": round(value, 1), "unit": "Mcells/s", "cores": 1, "kind": kind,
                             "sample": sample},
            "e2e": {"value": round(value, 1), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
    if w["kind"] == "serve":
        return {"impl": "reference", "unavailable": "the reference has no request loop (one kvs::MarchingCubes call "
                "at a time on the caller's thread); its per-request CPU cost is the uneven200 / sweep1024 reference "
                "arms"}
    planes = min(65, w["shape"][0]) if w["kind"] in ("fbm", "lattice") else w["shape"][0]
    args.mode = w.get("mode", 0)   # the workload's mode (duplicated, shared vertices, VertexNormal)
    if "pcts" in w:
        args.cpu_slab = cpu_slab_sample(args, planes)
        isos = workload_isos(w, args.cpu_slab.astype(np.float64).ravel())
    else:
        isos = w["isos"]
    vals = []
    sample = ""
    for i in range(args.warmup + args.steps):
        v, t, sample = run_cpu(args, threads, planes, isos)
        if i >= args.warmup:
            vals.append((v, t))
    value = statistics.median(v for v, _ in vals)
    ms = statistics.median(t for _, t in vals) * 1e3
    return {
        "impl": "reference", "metric": "Mcells/s", "value": round(value, 1), "unit": "Mcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["desc"], "sample": sample},
        "cpu_baseline": {"value": round(value, 1), "unit": "Mcells/s", "cores": min(threads, len(isos)),
                         "kind": "port",
                         "sample": sample + "; oracle/mc_oracle.c (C restatement of kvs::MarchingCubes, "
                         "-O3 -ffp-contract=off), one isovalue per thread"},
        "e2e": {"value": round(value, 1), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def host_cpu():
    """CPU model, host thread count and the CPU baselines' compiler, for the
    cpu_baseline entries."""
    import platform
    model = platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip() + " (" + platform.machine() + ")"
                break
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        gcc = subprocess.run(["gcc", "-dumpversion"], capture_output=True, text=True, timeout=10).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        gcc = "?"
    return {"cpu": model, "threads": os.cpu_count(),
            "compiler": f"gcc {gcc} -O3 -ffp-contract=off (oracle/mc_oracle.c); numpy {np.__version__} "
                        f"(oracle/*.py restatements)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sweep1024", choices=sorted(WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tune", action="store_true", help="run the launch-shape autotuner before measuring")
    ap.add_argument("--no-verify", action="store_true",
                    help="skip the check of the outputs against the oracle after the timed region")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif WORKLOADS[args.workload]["kind"] == "slice":
        line = run_slice(args, rank, world, local)
    elif WORKLOADS[args.workload]["kind"] == "cells":
        line = run_cells(args, rank, world, local)
        if rank == 0 and world == 1 and not args.no_cpu:
            v, t, sample, kind = run_cells_cpu(WORKLOADS[args.workload], reference=False)
            line["cpu_baseline"] = {"value": round(v, 1), "unit": "Mcells/s", "cores": 1, "kind": kind,
                                    "sample": sample + f"; {t:.1f} s on 1 host core"}
    elif WORKLOADS[args.workload]["kind"] == "ingest":
        line = run_ingest(args, rank, world, local)
    elif WORKLOADS[args.workload]["kind"] == "stl":
        line = run_stl(args, rank, world, local)
        mesh = line.pop("_sample_mesh")
        if rank == 0 and world == 1 and not args.no_cpu:
            v, t, nt = run_stl_cpu(mesh)
            line["cpu_baseline"] = {"value": round(v, 1), "unit": "Mtris/s", "cores": 1, "kind": "port",
                                    "sample": f"{nt} triangles of the first mesh, oracle/export.py (numpy "
                                              f"restatement of PolygonExporter<Stl> + Stl::write_binary), "
                                              f"{t:.1f} s on 1 host core"}
    elif WORKLOADS[args.workload]["kind"] == "stlascii":
        line = run_stl_ascii(args, rank, world, local)
        mesh = line.pop("_sample_mesh")
        if rank == 0 and world == 1 and not args.no_cpu:
            v, t, nt = run_stl_ascii_cpu(mesh)
            line["cpu_baseline"] = {"value": round(v, 3), "unit": "Mtris/s", "cores": 1, "kind": "port",
                                    "sample": f"{nt} triangles of the first mesh, oracle/export.py stl_ascii "
                                              f"(restatement of Stl::write_ascii), {t:.1f} s on 1 host core"}
    elif WORKLOADS[args.workload]["kind"] == "serve":
        line = run_serve(args, rank, world, local)
    elif WORKLOADS[args.workload]["kind"] == "batch":
        line = run_batch(args, rank, world, local)
        if rank == 0 and world == 1 and not args.no_cpu:
            v, t, sample = run_batch_cpu(args)
            line["cpu_baseline"] = {"value": round(v, 1), "unit": "Mcells/s", "cores": 1, "kind": "port",
                                    "sample": sample + f"; {t:.1f} s on 1 host core; oracle/mc_oracle.c"}
    else:
        line = run_ours(args, rank, world, local)
        if rank == 0 and world == 1 and not args.no_cpu:
            w = WORKLOADS[args.workload]
            planes = min(65, w["shape"][0]) if w["kind"] in ("fbm", "lattice") else w["shape"][0]
            isos = args.isos if w["kind"] in ("fbm", "lattice") else w["isos"] * 50
            v, t, sample = run_cpu(args, 1, planes, isos)
            line["cpu_baseline"] = {"value": round(v, 1), "unit": "Mcells/s", "cores": 1, "kind": "port",
                                    "sample": sample + f"; {t:.1f} s on 1 host core; oracle/mc_oracle.c"}
    if rank == 0 and line is not None:
        if isinstance(line.get("cpu_baseline"), dict):
            line["cpu_baseline"]["host"] = host_cpu()
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
