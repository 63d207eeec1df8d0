"""The KVS drop-in kvs::cuda::MarchingCubes (kvs_gb300/kvs/cuda) compiled
against the reference's own headers and linked with the reference's core
(oracle/_ref) and libkvsmc: it builds, satisfies the mapper plugin interface
(constructor form, setIsolevel/exec pipeline form, moduleName), and without a
GPU fails the reference's way (kvsMessageError, isSuccess() false, nullptr)."""
import os
import subprocess

import pytest

from oracle import ref

from .conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KVS_SRC = ref.REFERENCE_SOURCE


@pytest.mark.skipif(not (os.path.isdir(KVS_SRC) and ref.available()), reason="needs the reference sources")
def test_adapter_builds_and_fails_loudly_without_gpu(tmp_path):
    out = tmp_path / "adapter"
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "kvs_gb300", "kvs"), f"KVS_SRC={KVS_SRC}",
                        f"OUT={out}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / "demo"
    lib = os.path.join(ROOT, "kvs_gb300", "lib")
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-w", f"-I{KVS_SRC}", f"-I{os.path.join(ROOT, 'kvs_gb300')}",
                        f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "tests", "kvs_adapter", "main.cpp"),
                        str(out / "libkvsmc_kvs.a"), os.path.join(ROOT, "oracle", "_ref", "libkvsref.a"),
                        f"-L{lib}", "-lkvsmc", f"-Wl,-rpath,{lib}", "-lpthread", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if gpu_available():
        pytest.skip("checks the no-GPU behaviour")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert "ctor success=0 vertices=0" in r.stdout
    assert "exec success=0 returned=0 module=kvs::cuda::MarchingCubes" in r.stdout
    assert "null success=0 returned=0" in r.stdout
    assert "isosurface vertices=0 connections=0 module=kvs::cuda::Isosurface" in r.stdout
    assert "isosurface exec returned=0 vertices=0" in r.stdout
    assert "isosurface null returned=0" in r.stdout
    assert "Cannot create isosurfaces." in r.stdout + r.stderr
    assert "slice vertices=0 module=kvs::cuda::SlicePlane" in r.stdout
    assert "slice exec returned=0" in r.stdout
    assert "cells vertices=0 module=kvs::cuda::MarchingTetrahedra" in r.stdout
    assert "cells wrong type returned=0" in r.stdout
    assert "Input volume is not hexhedra-cell data." in r.stdout + r.stderr
    assert "cells isosurface vertices=0" in r.stdout
    assert "no CUDA device" in r.stdout + r.stderr


@pytest.mark.skipif(not (os.path.isdir(KVS_SRC) and ref.available()), reason="needs the reference sources")
def test_adapter_host_logic_matches_reference_in_process(tmp_path):
    """kvs::cuda::MarchingCubes and kvs::cuda::Isosurface beside the
    reference's kvs::MarchingCubes and kvs::Isosurface in one process, on twin
    volumes (Hydrogen 32^3, random float32 / int16 / uint8 / float64, a preset
    min/max, a constant volume), every mode, the constructor, pipeline and
    Isosurface forms: outputs, colour, types, bounding boxes, success flag and
    the volume's min/max cache bit for bit.  The C ABI is a test stand-in whose
    per-cell work is the oracle's (tests/kvs_adapter/oracle_backend.c), so this
    checks the drop-ins' host logic; the GPU tests check the C ABI itself."""
    out = tmp_path / "adapter"
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "kvs_gb300", "kvs"), f"KVS_SRC={KVS_SRC}",
                        f"OUT={out}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    stub = tmp_path / "libkvsmc.so"
    r = subprocess.run(["gcc", "-std=c11", "-D_POSIX_C_SOURCE=199309L", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        "-w", f"-I{os.path.join(ROOT, 'include')}",
                        os.path.join(ROOT, "tests", "kvs_adapter", "oracle_backend.c"), "-o", str(stub), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / "compare"
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-w", f"-I{KVS_SRC}", f"-I{os.path.join(ROOT, 'kvs_gb300')}",
                        f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "tests", "kvs_adapter", "compare.cpp"),
                        str(out / "libkvsmc_kvs.a"), os.path.join(ROOT, "oracle", "_ref", "libkvsref.a"),
                        f"-L{tmp_path}", "-lkvsmc", f"-Wl,-rpath,{tmp_path}", "-lpthread", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    last = r.stdout.strip().splitlines()[-1]
    cases = int(last.split()[0].split("=")[1])
    assert last.endswith("mismatches=0") and cases >= 150, last
