"""Generate mc_tables.h from the reference's MarchingCubesTable.cpp.

The marching-cubes triangle table (256 cases x up to 5 edge triples) and the
12-edge endpoint table are data that must be identical to the reference's
(Source/Core/Visualization/Mapper/MarchingCubesTable.cpp:16-290): the triangle
order inside a cell, and so the output order, comes from them.  This script
reads them from the reference source and writes them, plus the packed forms
the CUDA kernels use, into mc_tables.h, which is committed so that builds do
not need the reference.  tests/test_tables.py re-parses the reference (where
it is present) and checks the committed header entry for entry.

    python kvs_gb300/csrc/gen_mc_tables.py <KVS>/Source/Core/Visualization/Mapper/MarchingCubesTable.cpp

(or with KVS_SRC=<KVS>/Source in the environment and no argument).
"""
import os
import re
import sys


def parse_reference_tables(path):
    text = open(path).read()

    def block(name):
        m = re.search(name + r"\s*\[[^\]]*\]\s*\[[^\]]*\](?:\s*\[[^\]]*\])?\s*=\s*\{(.*?)\};", text, re.S)
        if not m:
            raise ValueError(f"{name} not found in {path}")
        return [int(v) for v in re.findall(r"-?\d+", m.group(1))]

    tri = block("TriangleID")
    vert = block("VertexID")
    if len(tri) != 256 * 16 or len(vert) != 12 * 2 * 3:
        raise ValueError("unexpected table sizes")
    tri_rows = [tri[16 * c:16 * c + 16] for c in range(256)]
    vert_rows = [[vert[6 * e:6 * e + 3], vert[6 * e + 3:6 * e + 6]] for e in range(12)]
    return tri_rows, vert_rows


def ntri(row):
    n = 0
    while n * 3 < 16 and row[3 * n] != -1:
        n += 1
    return n


def packed_emit_order(row):
    """Edges in emission order (e[i], e[i+2], e[i+1]) per triangle, 4 bits each,
    low nibble first; bits 60..63 hold the triangle count."""
    n = ntri(row)
    word = 0
    k = 0
    for t in range(n):
        for e in (row[3 * t], row[3 * t + 2], row[3 * t + 1]):
            word |= (e & 0xF) << (4 * k)
            k += 1
    word |= n << 60
    return word


def render(tri_rows, vert_rows):
    out = []
    out.append("/* Generated by gen_mc_tables.py from the reference's")
    out.append(" * Source/Core/Visualization/Mapper/MarchingCubesTable.cpp:16-290.")
    out.append(" * Do not edit by hand; tests/test_tables.py checks it against the reference. */")
    out.append("#ifndef KVSMC_MC_TABLES_H")
    out.append("#define KVSMC_MC_TABLES_H")
    out.append("#include <stdint.h>")
    out.append("")
    out.append("/* case -> edge triples, -1 terminated (TriangleID[256][16]) */")
    out.append("static const signed char MC_TRIANGLE_TABLE[256][16] = {")
    for c, row in enumerate(tri_rows):
        out.append("    {" + ", ".join(str(v) for v in row) + "},")
    out.append("};")
    out.append("")
    out.append("/* edge -> (start corner, end corner) offsets (VertexID[12][2][3]) */")
    out.append("static const signed char MC_EDGE_VERTEX[12][2][3] = {")
    for e, (a, b) in enumerate(vert_rows):
        out.append("    {{%d, %d, %d}, {%d, %d, %d}}," % (a[0], a[1], a[2], b[0], b[1], b[2]))
    out.append("};")
    out.append("")
    out.append("/* case -> number of triangles */")
    out.append("#define MC_NTRI_INIT { \\")
    n = [ntri(r) for r in tri_rows]
    for i in range(0, 256, 32):
        out.append("    " + ", ".join(str(v) for v in n[i:i + 32]) + ", \\")
    out.append("}")
    out.append("static const unsigned char MC_NTRI[256] = MC_NTRI_INIT;")
    out.append("")
    out.append("/* case -> edges in emission order (e[i], e[i+2], e[i+1]) as 4-bit fields,")
    out.append(" * low nibble first; bits 60..63 = triangle count */")
    out.append("#define MC_TRI_PACKED_INIT { \\")
    p = [packed_emit_order(r) for r in tri_rows]
    for i in range(0, 256, 4):
        out.append("    " + ", ".join("0x%016xull" % v for v in p[i:i + 4]) + ", \\")
    out.append("}")
    out.append("static const uint64_t MC_TRI_PACKED[256] = MC_TRI_PACKED_INIT;")
    out.append("")
    out.append("/* case -> bit mask of the edges its triangles use */")
    masks = []
    for r in tri_rows:
        m = 0
        for t in range(ntri(r)):
            for e in r[3 * t:3 * t + 3]:
                m |= 1 << e
        masks.append(m)
    out.append("#define MC_EDGE_MASK_INIT { \\")
    for i in range(0, 256, 16):
        out.append("    " + ", ".join("0x%03x" % v for v in masks[i:i + 16]) + ", \\")
    out.append("}")
    out.append("static const unsigned short MC_EDGE_MASK[256] = MC_EDGE_MASK_INIT;")
    out.append("")
    # edge -> packed endpoints: bits 0-2 start corner (x,y,z), bits 3-5 end corner
    out.append("/* edge -> start offset bits (x | y<<1 | z<<2) in bits 0..2, end offset in bits 3..5 */")
    ep = []
    for a, b in vert_rows:
        ep.append((a[0] | a[1] << 1 | a[2] << 2) | ((b[0] | b[1] << 1 | b[2] << 2) << 3))
    out.append("#define MC_EDGE_PACKED_INIT { " + ", ".join(str(v) for v in ep) + " }")
    out.append("static const unsigned char MC_EDGE_PACKED[12] = MC_EDGE_PACKED_INIT;")
    out.append("")
    out.append("#endif")
    return "\n".join(out) + "\n"


def main():
    if len(sys.argv) > 1:
        src = sys.argv[1]
    elif os.environ.get("KVS_SRC"):
        src = os.path.join(os.environ["KVS_SRC"], "Core", "Visualization", "Mapper", "MarchingCubesTable.cpp")
    else:
        sys.exit("usage: gen_mc_tables.py <path of MarchingCubesTable.cpp> (or set KVS_SRC to the KVS Source tree)")
    tri, vert = parse_reference_tables(src)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mc_tables.h")
    with open(dst, "w") as f:
        f.write(render(tri, vert))
    print("wrote", dst)


if __name__ == "__main__":
    main()
