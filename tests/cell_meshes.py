"""Seeded synthetic unstructured meshes for the marching-cells tests and fixtures.

A jittered grid of nx x ny x nz nodes split into hexahedra, tetrahedra (six
per hexahedron around its main diagonal), prisms (two per hexahedron) or
pyramids (six per hexahedron, apex at an added centre node, local node 0 the
apex as the pyramid mapper expects), and random meshes whose cells take any
nodes (every case of every table shows up).
"""
import numpy as np

TETRAHEDRA, HEXAHEDRA, PYRAMID, PRISM = 0, 1, 2, 3
NODES = {TETRAHEDRA: 4, HEXAHEDRA: 8, PYRAMID: 5, PRISM: 6}

# hexahedron corners: 0-3 on the lower z face, 4-7 above them
_CORNERS = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)])
_TETS = [(0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6)]
_PRISMS = [(0, 1, 2, 4, 5, 6), (0, 2, 3, 4, 6, 7)]
_FACES = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7)]


def grid(cell_type, nx, ny, nz, jitter=0.2, seed=0):
    """(coords float32[N, 3], connections uint32[C, nodes per cell])."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    xyz = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float64)
    xyz += rng.uniform(-jitter, jitter, xyz.shape)
    cz, cy, cx = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
    base = np.stack([cx.reshape(-1), cy.reshape(-1), cz.reshape(-1)], -1)
    c = base[:, None, :] + _CORNERS[None, :, :]
    hexa = (c[..., 0] + nx * (c[..., 1] + ny * c[..., 2])).astype(np.int64)      # [H, 8]
    if cell_type == HEXAHEDRA:
        conn = hexa
    elif cell_type == TETRAHEDRA:
        conn = hexa[:, _TETS].reshape(-1, 4)
    elif cell_type == PRISM:
        conn = hexa[:, _PRISMS].reshape(-1, 6)
    else:
        centre = xyz[hexa].mean(axis=1)
        ids = xyz.shape[0] + np.arange(hexa.shape[0])
        xyz = np.concatenate([xyz, centre])
        faces = hexa[:, _FACES]                                                   # [H, 6, 4]
        conn = np.concatenate([np.broadcast_to(ids[:, None, None], (hexa.shape[0], 6, 1)), faces],
                              axis=2).reshape(-1, 5)
    return xyz.astype(np.float32), np.ascontiguousarray(conn, np.uint32)


def random_mesh(cell_type, nnodes, ncells, seed=0):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(-4.0, 4.0, (nnodes, 3)).astype(np.float32)
    conn = rng.integers(0, nnodes, (ncells, NODES[cell_type])).astype(np.uint32)
    return xyz, conn


def sphere_values(xyz, centre=(2.3, 2.1, 1.9)):
    return np.sqrt(((xyz.astype(np.float64) - np.asarray(centre)) ** 2).sum(-1)).astype(np.float32)
