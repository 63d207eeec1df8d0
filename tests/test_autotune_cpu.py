"""The tuning table's host logic (size classes, resolution of a volume's
launch shape, validation, JSON files): pure host functions of libkvsmc.so,
no GPU needed."""
import numpy as np
import pytest

from kvs_gb300 import _abi
from kvs_gb300 import autotune as T


def test_size_classes():
    # cells = (nx-1)(ny-1)(nz-1); boundaries at 2^18, 2^21, 2^24, 2^27
    assert T.size_class(2, 2, 2) == 0
    assert T.size_class(64, 64, 64) == 0            # 63^3 < 2^18
    assert T.size_class(65, 65, 65) == 1            # 64^3 = 2^18
    assert T.size_class(129, 129, 128) == 1         # 128*128*127 < 2^21
    assert T.size_class(129, 129, 129) == 2         # 2^21
    assert T.size_class(257, 257, 257) == 3         # 2^24
    assert T.size_class(513, 513, 513) == 4         # 2^27
    assert T.size_class(1, 1000, 1000) == 0         # degenerate: no cells


def test_size_class_boundary_exact():
    assert T.size_class(4097, 1025, 2) == 2         # 2^22 cells
    assert T.size_class(4097, 4097, 9) == 4         # 2^27 cells


def test_builtin_rules():
    r = T.resolve([], np.float32, 101, 50, 50)      # 100 cells wide: two 128-cell rows per task
    assert r == {"rows": 2, "tasks_per_sm": 96, "ctas_per_sm": 0, "scan_threads": 256}
    assert T.resolve([], np.uint8, 257, 9, 9)["rows"] == 1    # 256 cells: tie -> one row
    assert T.resolve([], np.uint16, 301, 9, 9)["rows"] == 2   # 300 cells: 384 < 512 lanes
    assert T.resolve([], np.int16, 1024, 9, 9)["rows"] == 1   # 1023 cells


def test_table_overrides_only_its_class_and_dtype():
    table = [
        {"dtype": "float32", "size_class": 2, "rows": 1, "tasks_per_sm": 384, "ctas_per_sm": 0, "scan_threads": 64},
        {"dtype": "uint8", "size_class": 2, "rows": 0, "tasks_per_sm": 24, "ctas_per_sm": 1, "scan_threads": 0},
    ]
    r = T.resolve(table, np.float32, 201, 200, 200)          # class 2 float32
    assert r == {"rows": 1, "tasks_per_sm": 384, "ctas_per_sm": 0, "scan_threads": 64}
    r = T.resolve(table, np.uint8, 101, 400, 400)            # zero fields keep the rules (100 cells: 2 rows)
    assert r == {"rows": 2, "tasks_per_sm": 24, "ctas_per_sm": 1, "scan_threads": 256}
    assert T.resolve(table, np.float32, 50, 50, 50) == T.resolve([], np.float32, 50, 50, 50)   # class 0
    assert T.resolve(table, np.uint16, 201, 200, 200) == T.resolve([], np.uint16, 201, 200, 200)


@pytest.mark.parametrize("bad", [
    {"rows": 3}, {"rows": -1}, {"tasks_per_sm": -5}, {"ctas_per_sm": 65}, {"scan_threads": 100},
    {"scan_threads": 512}, {"size_class": 5}, {"size_class": -1}, {"dtype": "float64"}, {"dtype": "int32"},
])
def test_invalid_rows_are_refused(bad):
    row = {"dtype": "float32", "size_class": 1, "rows": 0, "tasks_per_sm": 0, "ctas_per_sm": 0, "scan_threads": 0}
    row.update(bad)
    with pytest.raises(_abi.KvsmcError):
        T.resolve([row], np.float32, 100, 100, 100)


def test_json_round_trip(tmp_path):
    table = [{"dtype": "int16", "size_class": 3, "rows": 2, "tasks_per_sm": 24, "ctas_per_sm": 0,
              "scan_threads": 128, "tuned_ms": 1.5, "default_ms": 1.8}]
    p = tmp_path / "t.json"
    T.save(str(p), table)
    assert T.load(str(p)) == table
    p.write_text('{"format": "other", "entries": []}')
    with pytest.raises(ValueError):
        T.load(str(p))
    bad = [dict(table[0], rows=7)]
    T.save(str(p), bad)
    with pytest.raises(_abi.KvsmcError):
        T.load(str(p))
