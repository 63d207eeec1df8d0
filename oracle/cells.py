"""CPU restatement of the reference's unstructured marching mappers.

TEST INFRASTRUCTURE ONLY: the checker for kvsmc_marching_cells_host and
kvsmc_slice_cells_host (imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline leg, never by kvs_gb300).  numpy,
vectorised over cells; pinned against the reference's own outputs in
tests/golden/cells.npz and tests/golden/slice_cells.npz.

Follows (Source/Core/Visualization/Mapper/):
  MarchingTetrahedra.cpp:155-236, MarchingHexahedra.cpp:143-230,
  MarchingPyramid.cpp:143-233, MarchingPrism.cpp:143-230
    - cells in order; local nodes = the cell's connections (hexahedra take
      connections 4-7 then 0-3, MarchingHexahedra.cpp:164-171);
    - case bit k set iff double(value of local node k) > isolevel
      (calculate_table_index); pyramid cases 10, 11, 20, 21 re-mapped to
      32-35 by the sign of E = (iso - A) D + B C (MarchingPyramid.cpp:293-315);
    - per triangle of the case, three edges (hexahedra and pyramids emit
      TriangleID[i], [i+2], [i+1]), a vertex per edge from interpolate_vertex:
      values clamped to the volume's [min, max] in double, ratio
      |(iso - v0) / (v1 - v0)|, c0 + ratio * float(c1 - c0) in double, rounded
      to float; normal (v1 - v0) x (v2 - v0) in float;
  UnstructuredVolumeObject.cpp:82-143 (GetMinMaxValues): with connections, a
    sequential scan from values[0] over values[conn[p]]; without, over the
    nodes.  Math::Min/Max (Utility/Math.h:27-50) keep the earlier value on
    ties and never take a NaN, so a NaN values[0] survives.
The per-type triangle and edge tables are read from the generated
kvs_gb300/csrc/cell_tables.h (a packed copy of the reference's tables).
"""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLES = os.path.join(os.path.dirname(HERE), "kvs_gb300", "csrc", "cell_tables.h")

TETRAHEDRA, HEXAHEDRA, PYRAMID, PRISM = 0, 1, 2, 3
NAMES = {TETRAHEDRA: "TETRA", HEXAHEDRA: "HEXA", PYRAMID: "PYRAMID", PRISM: "PRISM"}
NODES = {TETRAHEDRA: 4, HEXAHEDRA: 8, PYRAMID: 5, PRISM: 6}

_tables = None


def tables():
    """{cell_type: (ntri[case], edges[case, 5, 3] (emit order), edge_nodes[edge, 2])}"""
    global _tables
    if _tables is None:
        text = open(TABLES).read()
        out = {}
        for ct, name in NAMES.items():
            def grab(key):
                m = re.search(rf"#define CELL_{name}_{key}_INIT \{{(.*?)\}}", text)
                return [int(t.strip().rstrip("ull"), 0) for t in m.group(1).split(",")]
            ntri = np.array(grab("NTRI"), np.int64)
            words = grab("TRI")
            edges = np.zeros((len(words), 5, 3), np.int64)
            for c, w in enumerate(words):
                for t in range(5):
                    for s in range(3):
                        edges[c, t, s] = (w >> (12 * t + 4 * s)) & 15
            en = np.array([[e & 15, e >> 4] for e in grab("EDGE")], np.int64)
            out[ct] = (ntri, edges, en)
        _tables = out
    return _tables


def _seq_minmax(seq):
    """Math::Min/Max scan over seq (seq[0] is the start value)."""
    first = seq[0]
    if seq.dtype.kind == "f" and np.isnan(first):
        return float(first), float(first)
    ok = seq if seq.dtype.kind != "f" else seq[~np.isnan(seq)]
    lo, hi = ok.min(), ok.max()
    if seq.dtype.kind == "f":
        # ties: the first occurrence stays (only the sign of a zero shows)
        lo = ok[np.flatnonzero(ok == lo)[0]]
        hi = ok[np.flatnonzero(ok == hi)[0]]
    return float(lo), float(hi)


def minmax(values, connections, cell_type):
    """UnstructuredVolumeObject::updateMinMaxValues for veclen 1."""
    v = np.asarray(values).reshape(-1)
    conn = np.asarray(connections, np.int64).reshape(-1)
    if conn.size == 0:
        return _seq_minmax(v)
    return _seq_minmax(np.concatenate([v[:1], v[conn]]))


def _f64(v):
    # static_cast<double>: int64/uint64 round to nearest like the C conversion
    return np.asarray(v).astype(np.float64)


def marching_cells(cell_type, values, coords, connections, isolevel, minmax_values=None):
    """Duplicated-vertex extraction.  Returns dict(coords float32[9T],
    normals float32[3T], vmin, vmax, extracted)."""
    ct = int(cell_type)
    npc = NODES[ct]
    v = np.asarray(values).reshape(-1)
    xyz = np.asarray(coords, np.float32).reshape(-1, 3)
    conn = np.asarray(connections, np.int64).reshape(-1, npc)
    if minmax_values is None:
        vmin, vmax = minmax(v, conn, ct)
    else:
        vmin, vmax = float(minmax_values[0]), float(minmax_values[1])
    empty = dict(coords=np.zeros(0, np.float32), normals=np.zeros(0, np.float32), vmin=vmin, vmax=vmax,
                 extracted=False)
    if abs(vmin - vmax) < 1e-6:          # Math::Equal
        return empty
    empty["extracted"] = True
    if conn.shape[0] == 0:
        return empty
    nodes = conn[:, [4, 5, 6, 7, 0, 1, 2, 3]] if ct == HEXAHEDRA else conn
    vals = _f64(v[nodes])
    iso = float(isolevel)
    case = np.zeros(nodes.shape[0], np.int64)
    for k in range(npc):
        case |= (vals[:, k] > iso).astype(np.int64) << k
    if ct == PYRAMID:
        v1, v2, v3, v4 = vals[:, 1], vals[:, 2], vals[:, 3], vals[:, 4]
        with np.errstate(all="ignore"):
            A = (v1 + v2 + v3 + v4) / 4
            B = (-v1 + v2 + v3 - v4) / 4
            C = (-v1 - v2 + v3 + v4) / 4
            D = (v1 - v2 + v3 - v4) / 4
            E = (iso - A) * D + B * C
        case = np.where((case == 10) & (E < 0), 32, case)
        case = np.where((case == 11) & (E >= 0), 33, case)
        case = np.where((case == 20) & (E >= 0), 34, case)
        case = np.where((case == 21) & (E < 0), 35, case)
    ntri_t, edges_t, en = tables()[ct]
    ntri = ntri_t[case]
    T = int(ntri.sum())
    if T == 0:
        return empty
    cell = np.repeat(np.arange(nodes.shape[0]), ntri)
    first = np.repeat(np.cumsum(ntri) - ntri, ntri)
    k = np.arange(T) - first
    e = edges_t[case[cell], k]                        # [T, 3] edge ids
    n0 = nodes[cell[:, None], en[e, 0]]               # [T, 3] node ids
    n1 = nodes[cell[:, None], en[e, 1]]
    w0 = _f64(v[n0])
    w1 = _f64(v[n1])
    # Math::Clamp(a, lo, hi) = a <= lo ? lo : (a <= hi ? a : hi)
    w0 = np.where(w0 <= vmin, vmin, np.where(w0 <= vmax, w0, vmax))
    w1 = np.where(w1 <= vmin, vmin, np.where(w1 <= vmax, w1, vmax))
    with np.errstate(all="ignore"):
        r = np.abs((iso - w0) / (w1 - w0))
        c0 = xyz[n0]                                  # [T, 3, 3] float32
        c1 = xyz[n1]
        d = (c1 - c0).astype(np.float64)              # float difference
        p = (c0.astype(np.float64) + r[..., None] * d).astype(np.float32)
        u = p[:, 1] - p[:, 0]
        w = p[:, 2] - p[:, 0]
        nrm = np.stack([u[:, 1] * w[:, 2] - u[:, 2] * w[:, 1],
                        u[:, 2] * w[:, 0] - u[:, 0] * w[:, 2],
                        u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]], axis=1).astype(np.float32)
    return dict(coords=p.reshape(-1), normals=nrm.reshape(-1), vmin=vmin, vmax=vmax, extracted=True)


def min_max_coords(coords, connections):
    """UnstructuredVolumeObject::updateMinMaxCoords (UnstructuredVolumeObject.cpp:396-466):
    Math::Min(current, x) / Math::Max(current, x) per axis from the first
    connected node (all nodes without connections); a NaN x is taken, and the
    next value replaces it; on ties the later value wins."""
    xyz = np.asarray(coords, np.float32).reshape(-1, 3)
    conn = np.asarray(connections, np.int64).reshape(-1)
    seq = xyz if conn.size == 0 else np.concatenate([xyz[conn[:1]], xyz[conn]])
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    for ax in range(3):
        s = seq[:, ax]
        nan = np.flatnonzero(np.isnan(s))
        if nan.size and nan[-1] == s.size - 1:
            lo[ax] = hi[ax] = s[-1]
            continue
        t = s[nan[-1] + 1:] if nan.size else s
        mn, mx = t.min(), t.max()
        lo[ax] = t[np.flatnonzero(t == mn)[-1]]
        hi[ax] = t[np.flatnonzero(t == mx)[-1]]
    return lo, hi


# ---------------------------------------------------------------- SlicePlane

def _slice_value(a, b, r):
    """values[i0] + r * (values[i1] - values[i0]) with C++'s conversions per
    value type (SlicePlane.cpp:1043-1056), as the float ColorMap::at gets."""
    f32 = np.float32
    k = a.dtype
    if k in (np.int8, np.uint8, np.int16, np.uint16):
        d = b.astype(np.int32) - a.astype(np.int32)                 # int promotion
        return (a.astype(f32) + r * d.astype(f32)).astype(f32)
    if k == np.int32:
        d = (b.astype(np.int64) - a.astype(np.int64)).astype(np.uint32).view(np.int32)   # wraps
        return (a.astype(f32) + r * d.astype(f32)).astype(f32)
    if k == np.uint32:
        d = (b.astype(np.uint64) - a.astype(np.uint64)).astype(np.uint32)
        return (a.astype(f32) + r * d.astype(f32)).astype(f32)
    if k == np.int64:
        with np.errstate(over="ignore"):
            d = (b.view(np.uint64) - a.view(np.uint64)).view(np.int64)
        return (a.astype(f32) + r * d.astype(f32)).astype(f32)
    if k == np.uint64:
        with np.errstate(over="ignore"):
            d = b - a
        return (a.astype(f32) + r * d.astype(f32)).astype(f32)
    if k == np.float32:
        return (a + r * (b - a)).astype(f32)
    return (a + r.astype(np.float64) * (b - a)).astype(f32)       # double


def color_at(table, tf_min, tf_max, value):
    """ColorMap::at (ColorMap.cpp:1043-1054), RGBColor::Mix in float and the
    RGBColor(Vec3) rounding, vectorised; a NaN or out-of-range table position
    (undefined in the reference) takes entry 0."""
    f32 = np.float32
    table = np.asarray(table, np.uint8).reshape(-1, 3)
    res = table.shape[0]
    lo, hi = f32(tf_min), f32(tf_max)
    v = np.asarray(value, f32)
    v0 = np.where(v <= lo, lo, np.where(v <= hi, v, hi)).astype(f32)
    rr = f32(res - 1)
    with np.errstate(all="ignore"):
        pos = (((v0 - lo) / f32(hi - lo)).astype(f32) * rr).astype(f32)
    ok = (pos >= 0) & (pos <= rr)
    s0 = np.where(ok, pos, 0).astype(np.int64)
    s1 = np.minimum(s0 + 1, res - 1)
    t = np.where(ok, pos - s0.astype(f32), f32(0)).astype(f32)
    a = (table[s0].astype(f32) / f32(255)).astype(f32)
    b = (table[s1].astype(f32) / f32(255)).astype(f32)
    m = (a * (f32(1) - t)[:, None] + b * t[:, None]).astype(f32)
    m = np.where(m <= 0, f32(0), np.where(m <= 1, m, f32(1))).astype(f32)
    x = (m * f32(255)).astype(f32).astype(np.float64)
    return np.floor(x + 0.5).astype(np.uint8)


def slice_cells(cell_type, values, coords, connections, coefficients, table, tf_min, tf_max):
    """kvs::SlicePlane::extract_*_plane (SlicePlane.cpp:327-800) on an
    unstructured volume: (coords f32[9T], colors u8[9T], normals f32[3T])."""
    f32 = np.float32
    ct = int(cell_type)
    npc = NODES[ct]
    v = np.asarray(values).reshape(-1)
    xyz = np.asarray(coords, f32).reshape(-1, 3)
    conn = np.asarray(connections, np.int64).reshape(-1, npc)
    cf = np.asarray(coefficients, f32)
    empty = (np.zeros(0, f32), np.zeros(0, np.uint8), np.zeros(0, f32))
    if conn.shape[0] == 0:
        return empty

    def plane(p):   # ((a x + b y) + c z) + d in float
        ab = ((cf[0] * p[..., 0]).astype(f32) + (cf[1] * p[..., 1]).astype(f32)).astype(f32)
        return ((ab + (cf[2] * p[..., 2]).astype(f32)).astype(f32) + cf[3]).astype(f32)

    nodes = conn[:, [4, 5, 6, 7, 0, 1, 2, 3]] if ct == HEXAHEDRA else conn
    with np.errstate(all="ignore"):
        pv = plane(xyz).astype(f32)
    case = np.zeros(nodes.shape[0], np.int64)
    for k in range(npc):
        case |= (pv[nodes[:, k]] > 0).astype(np.int64) << k
    ntri_t, edges_t, en = tables()[ct]
    ntri = ntri_t[case]
    T = int(ntri.sum())
    if T == 0:
        return empty
    cell = np.repeat(np.arange(nodes.shape[0]), ntri)
    first = np.repeat(np.cumsum(ntri) - ntri, ntri)
    k = np.arange(T) - first
    e = edges_t[case[cell], k]
    if ct in (HEXAHEDRA, PYRAMID):
        e = e[:, [0, 2, 1]]          # the tables are packed in the mappers' [i], [i+2], [i+1] order
    n0 = nodes[cell[:, None], en[e, 0]]
    n1 = nodes[cell[:, None], en[e, 1]]
    p0, p1 = pv[n0], pv[n1]
    with np.errstate(all="ignore"):
        r = np.abs((p0 / (p1 - p0)).astype(f32)).astype(f32)
        s = (f32(1) - r).astype(f32)
        c0, c1 = xyz[n0], xyz[n1]
        pos = ((s[..., None] * c0).astype(f32) + (r[..., None] * c1).astype(f32)).astype(f32)
        val = _slice_value(v[n0], v[n1], r)
    rgb = color_at(table, tf_min, tf_max, val.reshape(-1)).reshape(T, 3, 3)
    with np.errstate(all="ignore"):
        u = pos[:, 2] - pos[:, 0]
        w = pos[:, 1] - pos[:, 0]
        nrm = -np.stack([u[:, 1] * w[:, 2] - u[:, 2] * w[:, 1],
                         u[:, 2] * w[:, 0] - u[:, 0] * w[:, 2],
                         u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]], axis=1).astype(f32)
    return pos.reshape(-1), rgb.reshape(-1), nrm.reshape(-1)
