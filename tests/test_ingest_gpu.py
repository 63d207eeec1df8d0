"""KVSML files loaded straight into device volumes (kvsmc_volume_load_kvsml)
against what the reference reader made of them (tests/golden/kvsml/): the
values bit for bit, the volume's min/max, and extraction from the loaded
volume equal to extraction from the same values uploaded."""
import os

import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import ingest

from .helpers import same_bits
from .test_ingest_cpu import KDIR, kvsml_cases


def load(ctx, c):
    p = os.path.join(KDIR, c["file"])
    return ingest.load_avs(ctx, p) if p.endswith(".fld") else ingest.load_kvsml(ctx, p)
from .test_stream_gpu import compare, extract_batch

pytestmark = pytest.mark.gpu


def test_loaded_volumes_match_reference_reader(kvsmc_ctx):
    cases, arr = kvsml_cases()
    for c in cases:
        dv, info = load(kvsmc_ctx, c)
        want = arr[c["name"]]
        got = dv.download()
        assert got.dtype == want.dtype and got.shape == want.shape, c["name"]
        assert same_bits(got, want), c["name"]
        assert (info["volume_min"], info["volume_max"]) == (c["vmin"], c["vmax"]), c["name"]
        assert dv.minmax() == (c["vmin"], c["vmax"]), c["name"]
        dv.free()


def test_extraction_from_loaded_volume(kvsmc_ctx):
    cases, arr = kvsml_cases()
    by_name = {c["name"]: c for c in cases}
    for name in ("f32_binary", "u8_binary", "i16_ascii", "f32_big", "f32_commas", "avs_f32", "avs_i16"):
        dv, info = load(kvsmc_ctx, by_name[name])
        up = _abi.DeviceVolume.upload(kvsmc_ctx, arr[name])
        lo, hi = info["volume_min"], info["volume_max"]
        ps = [_abi.make_params(lo + f * (hi - lo), 0, minmax=(lo, hi)) for f in (0.3, 0.55)]
        a = extract_batch(kvsmc_ctx, [dv] * 2, ps, _abi.PATH_AUTO)
        b = extract_batch(kvsmc_ctx, [up] * 2, ps, _abi.PATH_AUTO)
        for i in range(2):
            compare(a[i], b[i], f"{name} {i}")
        dv.free()
        up.free()


def test_short_or_missing_data_is_refused(kvsmc_ctx, tmp_path):
    text = open(os.path.join(KDIR, "f32_binary.kvsml")).read()
    raw = open(os.path.join(KDIR, "f32_binary_value.dat"), "rb").read()
    (tmp_path / "f32_binary_value.dat").write_bytes(raw[:-4])
    (tmp_path / "short.kvsml").write_text(text)
    with pytest.raises(_abi.KvsmcError):
        ingest.load_kvsml(kvsmc_ctx, tmp_path / "short.kvsml")
    (tmp_path / "missing.kvsml").write_text(text.replace("f32_binary_value.dat", "nothing.dat"))
    with pytest.raises(_abi.KvsmcError):
        ingest.load_kvsml(kvsmc_ctx, tmp_path / "missing.kvsml")
    fld = open(os.path.join(KDIR, "avs_u8.fld"), "rb").read()
    (tmp_path / "short.fld").write_bytes(fld[:-1])
    with pytest.raises(_abi.KvsmcError):
        ingest.load_avs(kvsmc_ctx, tmp_path / "short.fld")
    (tmp_path / "rect.fld").write_bytes(fld.replace(b"field  = uniform", b"field  = rectilinear"))
    with pytest.raises(_abi.KvsmcError):
        ingest.load_avs(kvsmc_ctx, tmp_path / "rect.fld")
    few = open(os.path.join(KDIR, "i8_ascii.kvsml")).read()
    start = few.index(">", few.index("<DataArray")) + 1
    (tmp_path / "few.kvsml").write_text(few[:start] + "1 2 3" + few[few.index("</DataArray>"):])
    with pytest.raises(_abi.KvsmcError):
        ingest.load_kvsml(kvsmc_ctx, tmp_path / "few.kvsml")
