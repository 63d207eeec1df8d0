"""libkvsmc.so on a host without a GPU: it loads, exports every symbol that
include/kvsmc.h declares, and refuses to run (no fallback) with clear statuses."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300.marching_cubes import MarchingCubes, PolygonObject, StructuredVolumeObject

from .conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "kvsmc.h")).read()
    return sorted(set(re.findall(r"\b(kvsmc_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(_abi.EXPORTS) == names


def test_status_strings():
    lib = _abi.load()
    for st in range(10):
        assert lib.kvsmc_status_string(st)
    assert lib.kvsmc_status_string(_abi.ERR_CAPACITY) == b"output buffer too small"


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_no_gpu_no_fallback():
    lib = _abi.load()
    h = C.c_void_p()
    assert lib.kvsmc_create(0, C.byref(h)) == _abi.ERR_NO_DEVICE
    with pytest.raises(_abi.KvsmcError):
        _abi.Context()
    s = _abi.Sizes()
    p = _abi.make_params(0.5, 0)
    x = np.zeros(64, np.float32)
    # the no-allocation entry point refuses before touching memory
    assert lib.kvsmc_extract_noalloc(x.ctypes.data, 8, 4, 4, 4, C.byref(p), None, 0, None, 0, None,
                                     C.byref(s)) in (_abi.ERR_NO_DEVICE, _abi.ERR_CUDA)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_mapper_reports_failure_like_the_reference(capsys):
    v = np.random.default_rng(0).random((4, 5, 6)).astype(np.float32)
    mc = MarchingCubes()
    assert mc.exec(StructuredVolumeObject(v)) is None
    assert not mc.isSuccess()
    assert "KVS ERROR" in capsys.readouterr().err


def test_mapper_argument_errors(capsys):
    mc = MarchingCubes()
    assert mc.exec(None) is None and not mc.isSuccess()
    assert mc.exec(PolygonObject()) is None and not mc.isSuccess()
    vol = StructuredVolumeObject(np.zeros((3, 3, 3), np.float32))
    vol.setVeclen(3)
    assert mc.exec(vol) is None and not mc.isSuccess()
    err = capsys.readouterr().err
    assert "Input object is NULL." in err and "not structured volume object" in err and "sclar" in err
