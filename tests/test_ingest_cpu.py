"""KVSML and AVS-field headers (kvsmc_kvsml_read_info, kvsmc_avs_read_info:
pure host functions) against what the reference readers
(StructuredVolumeObject::read; kvs::AVSField with the importer's rules) made
of the same files, tests/golden/kvsml/ (tests/golden/make_kvsml.py)."""
import json
import os

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import ingest

from .helpers import GOLDEN_DIR

KDIR = os.path.join(GOLDEN_DIR, "kvsml")


def kvsml_cases():
    return json.load(open(os.path.join(KDIR, "cases.json"))), np.load(os.path.join(KDIR, "expected.npz"))


def header(c):
    p = os.path.join(KDIR, c["file"])
    return ingest.read_avs_info(p) if p.endswith(".fld") else ingest.read_info(p)


def test_headers_match_reference_reader():
    cases, arr = kvsml_cases()
    assert len(cases) >= 20
    for c in cases:
        info = header(c)
        n = c["name"]
        assert info["dtype"] == np.dtype(c["dtype"]), n
        assert list(info["resolution"]) == c["resolution"] and info["veclen"] == c["veclen"], n
        assert info["uniform"], n
        assert np.array_equal(info["min_object_coord"], np.float32(c["min_obj"])), n
        assert np.array_equal(info["max_object_coord"], np.float32(c["max_obj"])), n
        if info["min_external_coord"] is not None:
            assert np.array_equal(info["min_external_coord"], np.float32(c["min_ext"])), n
            assert np.array_equal(info["max_external_coord"], np.float32(c["max_ext"])), n
        # the file's min/max where given (the reference then keeps them)
        if info["min_value"] is not None:
            assert info["min_value"] == c["vmin"], n
        if info["max_value"] is not None:
            assert info["max_value"] == c["vmax"], n
    fmt = {c["name"]: header(c)["format"] for c in cases}
    assert fmt["f32_ascii"] == "ascii" and fmt["f32_extascii"] == "external ascii" and fmt["f32_binary"] == "external binary"
    assert ingest.read_info(os.path.join(KDIR, "f32_big.kvsml"))["byte_swap"]


@pytest.mark.parametrize("text,status", [
    ("<KVSML><Object type='StructuredVolumeObject'></Object></KVSML>", _abi.ERR_INVALID_ARGUMENT),
    ("<KVSML><Object><StructuredVolumeObject grid_type='uniform'/></Object></KVSML>", _abi.ERR_INVALID_ARGUMENT),
    ("<KVSML><Object><StructuredVolumeObject grid_type='uniform' resolution='2 2'/></Object></KVSML>",
     _abi.ERR_INVALID_ARGUMENT),
    ("<KVSML><Object><StructuredVolumeObject grid_type='uniform' resolution='2 2 2'><Node><Value veclen='1'>"
     "<DataArray type='long'>1 2</DataArray></Value></Node></StructuredVolumeObject></Object></KVSML>",
     _abi.ERR_UNSUPPORTED_DTYPE),
    ("<KVSML><Object><StructuredVolumeObject grid_type='uniform' resolution='2 2 2'><Node><Value veclen='1'>"
     "<DataArray type='float' file='x.dat'/></Value></Node></StructuredVolumeObject></Object></KVSML>",
     _abi.ERR_INVALID_ARGUMENT),
    ("<KVSML><Object", _abi.ERR_INVALID_ARGUMENT),
])
def test_malformed_headers_are_refused(tmp_path, text, status):
    p = tmp_path / "bad.kvsml"
    p.write_text(text)
    with pytest.raises(_abi.KvsmcError) as e:
        ingest.read_info(p)
    assert e.value.status == status


def test_missing_file():
    with pytest.raises(_abi.KvsmcError):
        ingest.read_info("/nonexistent/volume.kvsml")
