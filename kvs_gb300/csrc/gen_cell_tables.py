"""Generate cell_tables.h from the reference's unstructured-grid marching tables.

The triangle tables and edge-endpoint tables of the tetrahedral, hexahedral,
pyramidal and prismatic marching mappers are data that must be identical to
the reference's (Source/Core/Visualization/Mapper/MarchingTetrahedraTable.cpp,
MarchingHexahedraTable.cpp, MarchingPyramidTable.cpp, MarchingPrismTable.cpp):
the triangle order inside a cell, and so the output order, comes from them.
This script reads them from the reference sources and writes their packed
forms into cell_tables.h, committed so that builds do not need the reference:
per case the triangle count and the edges of each triangle, already in the
order the mapper emits them (tetrahedra and prisms take TriangleID[i], [i+1],
[i+2]; hexahedra and pyramids [i], [i+2], [i+1]), and per edge its two local
node indices.

    python kvs_gb300/csrc/gen_cell_tables.py <KVS>/Source/Core/Visualization/Mapper

(or with KVS_SRC=<KVS>/Source in the environment and no argument).
"""
import os
import re
import sys

# (name, file, cases, row length, edges, swap the last two vertices)
CELLS = [
    ("TETRA", "MarchingTetrahedraTable.cpp", 16, 7, 6, False),
    ("HEXA", "MarchingHexahedraTable.cpp", 256, 16, 12, True),
    ("PYRAMID", "MarchingPyramidTable.cpp", 36, 13, 8, True),
    ("PRISM", "MarchingPrismTable.cpp", 64, 10, 9, False),
]


def parse(path, ncases, rowlen, nedges):
    text = open(path).read()

    def block(name):
        m = re.search(name + r"\s*\[[^\]]*\]\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", text, re.S)
        if not m:
            raise ValueError(f"{name} not found in {path}")
        return [int(v) for v in re.findall(r"-?\d+", re.sub(r"//[^\n]*", "", m.group(1)))]

    tri = block("TriangleID")
    vert = block("VertexID")
    if len(tri) != ncases * rowlen or len(vert) != nedges * 2:
        raise ValueError(f"{path}: unexpected table sizes {len(tri)} {len(vert)}")
    return [tri[rowlen * c:rowlen * c + rowlen] for c in range(ncases)], [vert[2 * e:2 * e + 2] for e in range(nedges)]


def pack(rows, swap):
    """Per case: (ntri, packed edges: 4 bits each, 3 per triangle, in emit order)."""
    out = []
    for row in rows:
        tris = []
        i = 0
        while i + 2 < len(row) and row[i] != -1:
            e0, e1, e2 = row[i], row[i + 1], row[i + 2]
            tris.append((e0, e2, e1) if swap else (e0, e1, e2))
            i += 3
        word = 0
        for t, (a, b, c) in enumerate(tris):
            word |= (a | (b << 4) | (c << 8)) << (12 * t)
        out.append((len(tris), word))
    return out


def main():
    if len(sys.argv) > 1:
        src = sys.argv[1]
    elif os.environ.get("KVS_SRC"):
        src = os.path.join(os.environ["KVS_SRC"], "Core", "Visualization", "Mapper")
    else:
        sys.exit("usage: gen_cell_tables.py <KVS Source/Core/Visualization/Mapper directory> (or set KVS_SRC)")
    lines = ["// cell_tables.h -- generated by gen_cell_tables.py from the reference's",
             "// unstructured-grid marching tables; do not edit.", "#pragma once", "#include <cstdint>", ""]
    for name, fn, ncases, rowlen, nedges, swap in CELLS:
        rows, verts = parse(os.path.join(src, fn), ncases, rowlen, nedges)
        packed = pack(rows, swap)
        lines.append(f"#define CELL_{name}_CASES {ncases}")
        lines.append(f"#define CELL_{name}_EDGES {nedges}")
        lines.append(f"#define CELL_{name}_NTRI_INIT {{ " + ", ".join(str(n) for n, _ in packed) + " }")
        lines.append(f"#define CELL_{name}_TRI_INIT {{ " + ", ".join(f"0x{w:x}ull" for _, w in packed) + " }")
        lines.append(f"#define CELL_{name}_EDGE_INIT {{ " + ", ".join(str(a | (b << 4)) for a, b in verts) + " }")
        lines.append("")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cell_tables.h")
    open(out, "w").write("\n".join(lines))
    print("wrote", out)


if __name__ == "__main__":
    main()
