"""The marching-cubes tables in kvs_gb300/csrc/mc_tables.h: entry for entry the
reference's MarchingCubesTable.cpp (where present), and internally consistent."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "kvs_gb300", "csrc", "mc_tables.h")
from oracle import ref as _ref

REF_TABLE = os.path.join(_ref.REFERENCE_SOURCE, "Core", "Visualization", "Mapper", "MarchingCubesTable.cpp")


def _header_tables():
    text = open(HEADER).read()

    def ints(name):
        m = re.search(name + r"[^=]*=\s*\{(.*?)\};", text, re.S)
        return [int(v, 0) for v in re.findall(r"-?0x[0-9a-f]+|-?\d+", m.group(1))]

    def macro(name):
        m = re.search(r"#define " + name + r" \{(.*?)\}\n", text, re.S)
        return [int(v, 0) for v in re.findall(r"0x[0-9a-f]+|\d+", m.group(1).replace("ull", ""))]

    tri = ints("MC_TRIANGLE_TABLE")
    vert = ints("MC_EDGE_VERTEX")
    return ([tri[16 * c:16 * c + 16] for c in range(256)], vert, macro("MC_NTRI_INIT"),
            macro("MC_TRI_PACKED_INIT"), macro("MC_EDGE_MASK_INIT"), macro("MC_EDGE_PACKED_INIT"))


def test_tables_consistent():
    tri, vert, ntri, packed, emask, epacked = _header_tables()
    assert len(tri) == 256 and len(vert) == 72 and len(ntri) == 256 and len(packed) == 256
    for c in range(256):
        n = 0
        while n < 5 and tri[c][3 * n] != -1:
            n += 1
        assert ntri[c] == n and packed[c] >> 60 == n
        m = 0
        for t in range(n):
            e0, e1, e2 = tri[c][3 * t], tri[c][3 * t + 1], tri[c][3 * t + 2]
            # emission order (e[i], e[i+2], e[i+1]) (MarchingCubes.cpp:206-208)
            assert (packed[c] >> (12 * t)) & 0xFFF == e0 | (e2 << 4) | (e1 << 8)
            m |= (1 << e0) | (1 << e1) | (1 << e2)
        assert emask[c] == m
    assert ntri[0] == 0 and ntri[255] == 0
    for e in range(12):
        a = vert[6 * e:6 * e + 3]
        b = vert[6 * e + 3:6 * e + 6]
        assert sum(abs(x - y) for x, y in zip(a, b)) == 1          # one axis
        assert epacked[e] == (a[0] | a[1] << 1 | a[2] << 2) | ((b[0] | b[1] << 1 | b[2] << 2) << 3)


@pytest.mark.skipif(not os.path.exists(REF_TABLE), reason="reference sources not present")
def test_tables_equal_reference():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "kvs_gb300", "csrc"))
    from gen_mc_tables import parse_reference_tables, render
    tri, vert = parse_reference_tables(REF_TABLE)
    assert open(HEADER).read() == render(tri, vert)


def test_vertex_triangle_bound():
    """The vertex normals keep fixed slots per vertex: a vertex lies on one
    cell edge, shared by at most 4 cells, and no case puts one edge into more
    than 5 of its triangles, so 4 x 5 slots hold every vertex's triangles."""
    tri = _header_tables()[0]
    most = 0
    for c in range(256):
        tris = [tri[c][3 * t:3 * t + 3] for t in range(5) if tri[c][3 * t] != -1]
        for e in range(12):
            most = max(most, sum(e in t for t in tris))
    assert most == 5
    src = open(os.path.join(ROOT, "kvs_gb300", "csrc", "mc_gather.cu")).read()
    m = re.search(r"constexpr uint32_t kVnMaxInc = (\d+);", src)
    assert m and int(m.group(1)) == 4 * most
