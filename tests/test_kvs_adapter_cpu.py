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
