"""Seeded synthetic structured volumes (the benchmark workloads' stand-ins).

No public dataset is named for this path; these generators produce fields
with the shapes, dtypes and value distributions of the workloads:

  gaussian_blobs       sum of isotropic Gaussians + uniform noise (float32)
  fbm                  fractal Brownian motion of 3-D gradient noise in [0, 1]
  ellipsoid_phantom    nested rotated ellipsoidal shells + Gaussian noise
  box_filtered_noise   white noise low-passed by a box filter per axis
  lattice_noise        white noise on a coarse lattice, trilinearly interpolated

All return arrays shaped (nz, ny, nx) (x fastest, as the mapper expects).
They run with torch on any device, so the large fields are made on the GPU
in z-slabs; small ones on the CPU feed the parity tests.
"""
import math

import numpy as np
import torch


def _dtype_range(dtype):
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return 0.0, 1.0
    info = np.iinfo(dt)
    return float(info.min), float(info.max)


def _cast(field, dtype):
    """Clamp and round a float field into an integer dtype (or cast to float)."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return field.to(getattr(torch, dt.name))
    lo, hi = _dtype_range(dt)
    f = torch.clamp(torch.round(field.double()), lo, hi)
    tmap = {"int8": torch.int8, "uint8": torch.uint8, "int16": torch.int16, "uint16": torch.uint16,
            "int32": torch.int32, "uint32": torch.uint32, "int64": torch.int64, "uint64": torch.uint64}
    return f.to(tmap[dt.name])


def gaussian_blobs(shape, nblobs=4, sigma=(8.0, 24.0), noise=0.01, seed=0, device="cpu"):
    """Sum of `nblobs` exp(-d^2 / 2 sigma^2) (amplitude 1), centres uniform in
    the box, sigma uniform in `sigma`, plus uniform noise in [-noise, noise]."""
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, 1.0, size=(nblobs, 3)) * (np.array([nx, ny, nz]) - 1)
    sig = rng.uniform(sigma[0], sigma[1], size=nblobs)
    gen = torch.Generator(device=device).manual_seed(seed)
    x = torch.arange(nx, device=device, dtype=torch.float32)
    y = torch.arange(ny, device=device, dtype=torch.float32)
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=device)
    slab = max(1, (1 << 24) // max(1, nx * ny))
    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        z = torch.arange(z0, z1, device=device, dtype=torch.float32)
        f = torch.zeros((z1 - z0, ny, nx), dtype=torch.float32, device=device)
        for (cx, cy, cz), s in zip(centres, sig):
            dz = (z - float(cz)) ** 2
            dy = (y - float(cy)) ** 2
            dx = (x - float(cx)) ** 2
            d2 = dz[:, None, None] + dy[None, :, None] + dx[None, None, :]
            f += torch.exp(-d2 / float(2.0 * s * s))
        f += (torch.rand(f.shape, generator=gen, device=device) * 2.0 - 1.0) * noise
        out[z0:z1] = f
    return out


def _hash3(ix, iy, iz, seed):
    """Integer hash of lattice points (int64 tensors) -> int64 in [0, 2^31)."""
    h = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
    h = h & 0x7FFFFFFF
    h = (h ^ (h >> 13)) * 1274126177
    h = h & 0x7FFFFFFF
    h = h ^ (h >> 16)
    return h


_GRADS = torch.tensor([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0],
                       [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                       [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1]], dtype=torch.float32)


def _gradient_noise(px, py, pz, seed):
    """3-D gradient (Perlin-style) noise at float coordinates (broadcastable)."""
    grads = _GRADS.to(px.device)
    fx, fy, fz = torch.floor(px), torch.floor(py), torch.floor(pz)
    tx, ty, tz = px - fx, py - fy, pz - fz
    ix, iy, iz = fx.long(), fy.long(), fz.long()

    def fade(t):
        return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)

    ux, uy, uz = fade(tx), fade(ty), fade(tz)
    acc = None
    for cz in (0, 1):
        for cy in (0, 1):
            for cx in (0, 1):
                g = grads[_hash3(ix + cx, iy + cy, iz + cz, seed) % 12]
                d = g[..., 0] * (tx - cx) + g[..., 1] * (ty - cy) + g[..., 2] * (tz - cz)
                w = (ux if cx else 1.0 - ux) * (uy if cy else 1.0 - uy) * (uz if cz else 1.0 - uz)
                acc = d * w if acc is None else acc + d * w
    return acc


def fbm(shape, octaves=5, base_freq=1.0 / 128.0, gain=0.5, lacunarity=2.0, seed=0, device="cpu",
        out=None):
    """Fractal Brownian motion of gradient noise, rescaled to [0, 1] (float32)."""
    nz, ny, nx = shape
    if out is None:
        out = torch.empty((nz, ny, nx), dtype=torch.float32, device=device)
    x = torch.arange(nx, device=device, dtype=torch.float32)
    y = torch.arange(ny, device=device, dtype=torch.float32)
    # elements per generated slab: large on a GPU (fewer launches), small on the CPU
    slab = max(1, (1 << (26 if str(device).startswith("cuda") else 22)) // max(1, nx * ny))
    for z0 in range(0, nz, slab):
        z1 = min(nz, z0 + slab)
        z = torch.arange(z0, z1, device=device, dtype=torch.float32)
        pz, py, px = z[:, None, None], y[None, :, None], x[None, None, :]
        pz, py, px = torch.broadcast_tensors(pz, py, px)
        f = torch.zeros(pz.shape, dtype=torch.float32, device=device)
        amp, freq = 1.0, base_freq
        for o in range(octaves):
            f += amp * _gradient_noise(px * freq, py * freq, pz * freq, seed * 131 + o)
            amp *= gain
            freq *= lacunarity
        out[z0:z1] = f
    lo, hi = out.min(), out.max()
    out.sub_(lo).div_(hi - lo)
    out.clamp_(0.0, 1.0)
    return out


def ellipsoid_phantom(shape, dtype, seed=0, device="cpu"):
    """3-6 nested ellipsoidal shells with random axes and rotations; shell
    values uniform over the dtype's range (floats: [0, 1]); Gaussian noise with
    sigma = 2% of the range; clamped and rounded for integer dtypes."""
    nz, ny, nx = shape
    rng = np.random.default_rng(seed)
    lo, hi = _dtype_range(dtype)
    nshell = int(rng.integers(3, 7))
    centre = np.array([nx, ny, nz], float) / 2.0 + rng.uniform(-0.1, 0.1, 3) * np.array([nx, ny, nz])
    out = torch.full((nz, ny, nx), lo + 0.0 * (hi - lo), dtype=torch.float64, device=device)
    x = torch.arange(nx, device=device, dtype=torch.float64) - centre[0]
    y = torch.arange(ny, device=device, dtype=torch.float64) - centre[1]
    z = torch.arange(nz, device=device, dtype=torch.float64) - centre[2]
    Z, Y, X = torch.meshgrid(z, y, x, indexing="ij")
    base = 0.45 * np.array([nx, ny, nz], float)
    for s in range(nshell):
        frac = 1.0 - s / (nshell + 0.5)
        axes = base * frac * rng.uniform(0.6, 1.0, 3)
        a, b, c = rng.uniform(0, 2 * math.pi, 3)
        ca, sa, cb, sb, cc, sc = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
        R = np.array([[ca * cb, ca * sb * sc - sa * cc, ca * sb * cc + sa * sc],
                      [sa * cb, sa * sb * sc + ca * cc, sa * sb * cc - ca * sc],
                      [-sb, cb * sc, cb * cc]])
        u = R[0, 0] * X + R[1, 0] * Y + R[2, 0] * Z
        v = R[0, 1] * X + R[1, 1] * Y + R[2, 1] * Z
        w = R[0, 2] * X + R[1, 2] * Y + R[2, 2] * Z
        inside = (u / axes[0]) ** 2 + (v / axes[1]) ** 2 + (w / axes[2]) ** 2 <= 1.0
        val = float(rng.uniform(lo, hi))
        out[inside] = val
    gen = torch.Generator(device=device).manual_seed(seed)
    out += torch.randn(out.shape, generator=gen, device=device, dtype=torch.float64) * (0.02 * (hi - lo))
    if np.dtype(dtype).kind == "f":
        out.clamp_(lo, hi)
    return _cast(out, dtype)


def _box_wide(f, dim, taps):
    """Box filter of odd width `taps` along one dimension (edges replicated),
    through a running sum."""
    h = taps // 2
    n = f.shape[dim]
    g = torch.cat([f.narrow(dim, 0, 1).expand(*[h if d == dim else -1 for d in range(f.dim())]), f,
                   f.narrow(dim, n - 1, 1).expand(*[h if d == dim else -1 for d in range(f.dim())])], dim)
    c = torch.cumsum(g, dim)
    del g
    zero = torch.zeros_like(c.narrow(dim, 0, 1))
    c = torch.cat([zero, c], dim)
    return (c.narrow(dim, taps, n) - c.narrow(dim, 0, n)) / taps


def box_filtered_noise(shape, dtype=np.uint16, seed=0, device="cpu", taps=3):
    """White noise uniform over the dtype's range, box-filtered (`taps` taps,
    odd, edge replicated) along x, y and z, rounded back to the dtype."""
    nz, ny, nx = shape
    lo, hi = _dtype_range(dtype)
    gen = torch.Generator(device=device).manual_seed(seed)
    f = torch.rand((nz, ny, nx), generator=gen, device=device, dtype=torch.float32) * (hi - lo) + lo
    for dim in (2, 1, 0):
        n = f.shape[dim]
        if n < 2:
            continue
        if taps == 3:
            idx = torch.arange(n, device=device)
            left = f.index_select(dim, torch.clamp(idx - 1, 0, n - 1))
            right = f.index_select(dim, torch.clamp(idx + 1, 0, n - 1))
            f = (left + f + right) / 3.0
        else:
            f = _box_wide(f, dim, taps)
    return _cast(f, dtype)


def lattice_noise(shape, dtype=np.uint16, seed=0, device="cpu", spacing=32):
    """White noise uniform over the dtype's range on a lattice of the given
    spacing (in cells), trilinearly interpolated to the full grid (a low-pass
    of white noise whose isosurfaces cross about 2/spacing of the cells per
    isovalue), rounded back to the dtype."""
    nz, ny, nx = shape
    lo, hi = _dtype_range(dtype)
    gen = torch.Generator(device=device).manual_seed(seed)
    cz, cy, cx = ((n - 1 + spacing - 1) // spacing + 1 for n in shape)
    c = torch.rand((1, 1, cz, cy, cx), generator=gen, device=device, dtype=torch.float32) * (hi - lo) + lo
    # sample the coarse grid at the fine nodes (node i at coarse coordinate i / spacing)
    f = torch.empty((nz, ny, nx), dtype=torch.float32, device=device)
    zs = torch.arange(nz, device=device, dtype=torch.float32) / spacing
    ys = torch.arange(ny, device=device, dtype=torch.float32) / spacing
    xs = torch.arange(nx, device=device, dtype=torch.float32) / spacing
    cc = c[0, 0]
    y0 = ys.floor().long().clamp(max=cy - 2)
    x0 = xs.floor().long().clamp(max=cx - 2)
    wy = (ys - y0.float())[:, None]
    wx = (xs - x0.float())[None, :]
    for z in range(nz):
        z0 = min(int(zs[z].floor().item()), cz - 2)
        wz = float(zs[z].item()) - z0
        plane = cc[z0] * (1.0 - wz) + cc[z0 + 1] * wz
        a = plane[y0][:, x0] * (1.0 - wx) + plane[y0][:, x0 + 1] * wx
        b = plane[y0 + 1][:, x0] * (1.0 - wx) + plane[y0 + 1][:, x0 + 1] * wx
        f[z] = a * (1.0 - wy) + b * wy
    return _cast(f, dtype)


def to_numpy(t):
    """Host numpy copy of a generated tensor."""
    t = t.cpu()
    if t.dtype == torch.uint16:
        return t.view(torch.int16).numpy().view(np.uint16)
    if t.dtype == torch.uint32:
        return t.view(torch.int32).numpy().view(np.uint32)
    if t.dtype == torch.uint64:
        return t.view(torch.int64).numpy().view(np.uint64)
    return t.numpy()
