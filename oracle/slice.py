"""CPU restatement of the reference's SlicePlane on structured volumes.

TEST INFRASTRUCTURE ONLY: the checker for kvsmc_slice_plane and
kvsmc_slice_extract_device (imported by tests/, never by kvs_gb300).  numpy,
vectorised over cells; pinned against the reference's own outputs in
tests/golden/slice.npz and, where the reference is built, against it live.

Follows Source/Core/Visualization/Mapper/SlicePlane.cpp:
  extract_plane (structured) :157-281
    - cells in z, y, x order (x fastest); case bit k set iff the plane
      equation at corner k is > 0 (calculate_table_index :802-818, corners
      0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0), 4-7 the same at z+1); cases 0
      and 255 skipped;
    - per triangle the edges TriangleID[i], [i+2], [i+1]; the endpoints are
      the cell's corner plus VertexID[e][0] and VertexID[e][1] as floats;
    - vertex = scale_coord(interpolate_vertex(v0, v1)) with
      interpolate_vertex :986-996 (float ratio |p0 / (p1 - p0)|,
      (1 - r) v0 + r v1 in float) and scale_coord (coord + min) * scale,
      scale = (max - min) / ncells in float;
    - per vertex the value values[i0] + r (values[i1] - values[i0]) in the
      value type's arithmetic (interpolate_value :1007-1030) and its colour
      ColorMap::at;
    - normal -(vertex2 - vertex0) x (vertex1 - vertex0) in float;
  substitute_plane_equation :949-979: ((a x + b y) + c z) + d in float.
Tables come from kvs_gb300/csrc/mc_tables.h (a generated copy of the
reference's MarchingCubesTable); colour and value arithmetic are shared with
the unstructured restatement in oracle/cells.py.
"""
import os
import re

import numpy as np

from . import cells as _cells

HERE = os.path.dirname(os.path.abspath(__file__))
MC_TABLES = os.path.join(os.path.dirname(HERE), "kvs_gb300", "csrc", "mc_tables.h")

# corner k of a cell as (dx, dy, dz) (MarchingCubes.cpp:187-194 / SlicePlane.cpp:808-815)
CORNERS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                    (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], np.int64)

_tables = None


def mc_tables():
    """(triangle table int8[256, 16], edge endpoints int64[12, 2, 3]): the
    reference's MarchingCubesTable::TriangleID and VertexID
    (MarchingCubesTable.cpp:16-290), read from the generated header."""
    global _tables
    if _tables is None:
        text = open(MC_TABLES).read()

        def block(name):
            m = re.search(name + r"\[[^=]*=\s*\{(.*?)\};", text, re.S)
            return np.array([int(t) for t in re.findall(r"-?\d+", m.group(1))], np.int64)

        tri = block("MC_TRIANGLE_TABLE").reshape(256, 16)
        ev = block("MC_EDGE_VERTEX").reshape(12, 2, 3)
        _tables = (tri, ev)
    return _tables


def _plane(cf, x, y, z):
    """substitute_plane_equation (SlicePlane.cpp:949-979) in float."""
    f32 = np.float32
    ab = ((cf[0] * x).astype(f32) + (cf[1] * y).astype(f32)).astype(f32)
    return ((ab + (cf[2] * z).astype(f32)).astype(f32) + cf[3]).astype(f32)


def slice_plane(values, coefficients, table, tf_min, tf_max, min_coord=None, max_coord=None):
    """SlicePlane::extract_plane on a structured volume (SlicePlane.cpp:157-281).
    values: array [nz, ny, nx] of any of the ten value types.  Returns
    (coords f32[9T], colors u8[9T], normals f32[3T]) as the reference's
    SlicePlane sets them; min_coord/max_coord default to the uniform
    volume's bounding box (0 and dims - 1)."""
    f32 = np.float32
    v = np.asarray(values)
    nz, ny, nx = v.shape
    cx, cy, cz = nx - 1, ny - 1, nz - 1
    empty = (np.zeros(0, f32), np.zeros(0, np.uint8), np.zeros(0, f32))
    if min(cx, cy, cz) <= 0:
        return empty
    cf = np.asarray(coefficients, f32)
    lo = np.zeros(3, f32) if min_coord is None else np.asarray(min_coord, f32)
    hi = np.array([cx, cy, cz], f32) if max_coord is None else np.asarray(max_coord, f32)
    scale = ((hi - lo).astype(f32) / np.array([cx, cy, cz], f32)).astype(f32)
    tri_t, ev = mc_tables()
    ntri_t = (tri_t >= 0).sum(1) // 3

    zz, yy, xx = np.meshgrid(np.arange(nz, dtype=f32), np.arange(ny, dtype=f32), np.arange(nx, dtype=f32),
                             indexing="ij")
    with np.errstate(all="ignore"):
        pv = _plane(cf, xx, yy, zz)                                  # [nz, ny, nx]
    pos = pv > 0
    case = np.zeros((cz, cy, cx), np.int64)
    for k, (dx, dy, dz) in enumerate(CORNERS):
        case |= pos[dz:dz + cz, dy:dy + cy, dx:dx + cx].astype(np.int64) << k
    case = case.reshape(-1)
    ntri = np.where((case == 0) | (case == 255), 0, ntri_t[case])
    T = int(ntri.sum())
    if T == 0:
        return empty
    cell = np.repeat(np.arange(case.size), ntri)
    k = np.arange(T) - np.repeat(np.cumsum(ntri) - ntri, ntri)
    e = tri_t[case[cell][:, None], 3 * k[:, None] + np.array([0, 2, 1])]        # [T, 3]
    base = np.stack([cell % cx, (cell // cx) % cy, cell // (cx * cy)], axis=1)  # x, y, z
    a = base[:, None, :] + ev[e, 0]                                          # [T, 3, 3] integer corners
    b = base[:, None, :] + ev[e, 1]
    vf = v.reshape(-1)
    ia = a[..., 0] + a[..., 1] * nx + a[..., 2] * nx * ny
    ib = b[..., 0] + b[..., 1] * nx + b[..., 2] * nx * ny
    p0, p1 = pv.reshape(-1)[ia], pv.reshape(-1)[ib]
    with np.errstate(all="ignore"):
        r = np.abs((p0 / (p1 - p0)).astype(f32)).astype(f32)
        s = (f32(1) - r).astype(f32)
        vert = ((s[..., None] * a.astype(f32)).astype(f32) + (r[..., None] * b.astype(f32)).astype(f32)).astype(f32)
        vert = ((vert + lo).astype(f32) * scale).astype(f32)
        val = _cells._slice_value(vf[ia], vf[ib], r)
    rgb = _cells.color_at(table, tf_min, tf_max, val.reshape(-1)).reshape(T, 3, 3)
    with np.errstate(all="ignore"):
        u = vert[:, 2] - vert[:, 0]
        w = vert[:, 1] - vert[:, 0]
        nrm = -np.stack([u[:, 1] * w[:, 2] - u[:, 2] * w[:, 1],
                         u[:, 2] * w[:, 0] - u[:, 0] * w[:, 2],
                         u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]], axis=1).astype(f32)
    return vert.reshape(-1), rgb.reshape(-1), nrm.reshape(-1)
