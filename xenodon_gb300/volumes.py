"""Seeded synthetic volumes standing in for the reference's datasets.

The reference renders a CT scan of the Stanford bunny (512x361x512) and TNG
gas fields (1024^3, 2048^3) prepared by tools/make-bunny-volume.py and
tools/make-tng-volume.py; none of that data is available, so these generators
produce volumes of the same shapes and value distributions.  All voxels are
RGBA8 with alpha 255 (as tools/make-bunny-volume.py:48 writes), "zeroed" means
RGB = 0, and arrays are laid out (dz, dy, dx, 4), x fastest, like
src/model/Grid.h:50-52.

Randomness comes from integer hashes of voxel coordinates and a seed, so a
volume is the same whichever torch device evaluates it (up to float rounding in
the smooth noise).
"""
from __future__ import annotations

import math

import numpy as np
import torch

_M32 = 0xFFFFFFFF


def _hash32(a: torch.Tensor) -> torch.Tensor:
    """Thomas Wang's 32-bit integer hash on int64 tensors holding u32 values."""
    a = ((a ^ 61) ^ (a >> 16)) & _M32
    a = (a + (a << 3)) & _M32
    a = a ^ (a >> 4)
    a = (a * 0x27D4EB2D) & _M32
    a = a ^ (a >> 15)
    return a


def _uniform(x, y, z, seed: int, salt: int) -> torch.Tensor:
    """Uniform [0, 1) per integer coordinate."""
    h = _hash32((x * 73856093) & _M32)
    h = _hash32(h ^ ((y * 19349663) & _M32))
    h = _hash32(h ^ ((z * 83492791) & _M32))
    h = _hash32(h ^ ((seed * 2654435761 + salt * 40503) & _M32))
    return h.to(torch.float64) / 4294967296.0


def _device(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def blobs(n: int = 128, seed: int = 0, count: int = 16) -> np.ndarray:
    """16 isotropic Gaussian blobs in an n^3 grid (the 128^3 DDA workload).

    Centres uniform in [0.2, 0.8]^3 of the extent, sigma uniform in
    [0.03, 0.1] of the extent, per-blob RGB uniform in [0, 255]; the colours
    are summed and clamped to 255 per channel, and voxels whose largest channel
    is below 8 are zeroed (about 80% of the volume is empty)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, (count, 3)) * n
    sigmas = rng.uniform(0.03, 0.1, count) * n
    colours = rng.integers(0, 256, (count, 3)).astype(np.float64)
    c = (np.arange(n) + 0.5)
    acc = np.zeros((n, n, n, 3), np.float64)
    for k in range(count):
        gz = np.exp(-((c - centres[k, 2]) ** 2) / (2 * sigmas[k] ** 2))
        gy = np.exp(-((c - centres[k, 1]) ** 2) / (2 * sigmas[k] ** 2))
        gx = np.exp(-((c - centres[k, 0]) ** 2) / (2 * sigmas[k] ** 2))
        w = gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
        acc += w[..., None] * colours[k]
    rgb = np.minimum(np.floor(acc), 255).astype(np.uint8)
    rgb[rgb.max(axis=3) < 8] = 0
    out = np.empty((n, n, n, 4), np.uint8)
    out[..., :3] = rgb
    out[..., 3] = 255
    return out


def ct_shell(dx: int = 512, dy: int = 361, dz: int = 512, seed: int = 1, device=None) -> np.ndarray:
    """CT-scan-shaped volume (the 512x361x512 bunny stand-in).

    A closed ellipsoidal shell with semi-axes 0.40/0.35/0.30 of the largest
    extent and a thickness of 3-6 voxels, its radius perturbed by 3-octave
    value noise of amplitude 0.05; the interior holds gray N(90, 20) clamped to
    [1, 255] at 20% of its voxels; the background is 0.  The normal variate is
    the sum of twelve hashed uniforms less 6 (Irwin-Hall), added one at a time
    in float32, and the rest is integer hashing and single IEEE operations,
    so the bytes are the same on every host and device."""
    dev = _device(device)
    ext = float(max(dx, dy, dz))
    a, b, c = 0.40 * ext, 0.35 * ext, 0.30 * ext
    cx, cy, cz = dx / 2.0, dy / 2.0, dz / 2.0
    mean_axis = (a + b + c) / 3.0
    f32 = torch.float32
    xs = torch.arange(dx, device=dev, dtype=f32) + 0.5
    ys = torch.arange(dy, device=dev, dtype=f32) + 0.5
    # smooth fields over the whole volume are evaluated slab by slab with the
    # lattice origin fixed at 0, so slabs join seamlessly
    out = np.empty((dz, dy, dx, 4), np.uint8)
    slab = max(1, (1 << 23) // (dx * dy))
    xi = torch.arange(dx, device=dev, dtype=torch.int64)[None, None, :]
    yi = torch.arange(dy, device=dev, dtype=torch.int64)[None, :, None]
    for z0 in range(0, dz, slab):
        z1 = min(dz, z0 + slab)
        zs = torch.arange(z0, z1, device=dev, dtype=f32) + 0.5
        X, Y, Z = ((xs - cx) / a)[None, None, :], ((ys - cy) / b)[None, :, None], ((zs - cz) / c)[:, None, None]
        rho = torch.sqrt(X * X + Y * Y + Z * Z)
        noise = (_noise_fixed(xs, ys, zs, ext / 8, seed, 1) + 0.5 * _noise_fixed(xs, ys, zs, ext / 16, seed, 2)
                 + 0.25 * _noise_fixed(xs, ys, zs, ext / 32, seed, 3)) / 1.75
        rho = rho * (1.0 + 0.05 * noise)
        thick = 3.0 + 3.0 * (0.5 + 0.5 * _noise_fixed(xs, ys, zs, ext / 12, seed, 4))
        dist = (rho - 1.0) * mean_axis  # signed distance in voxels, approximately
        shell = dist.abs() <= thick / 2
        inner = dist < -thick / 2
        zi = torch.arange(z0, z1, device=dev, dtype=torch.int64)[:, None, None]
        lin = (xi + dx * (yi + dy * zi)) & _M32
        h1 = _hash32(lin ^ ((seed * 0x9E3779B1 + 5) & _M32))
        u1 = h1.to(f32) / 4294967296.0
        h, gauss = h1, None
        for k in range(12):
            h = _hash32(h ^ ((0x68E31DA4 + 0x1B56C4E9 * k) & _M32))
            u = h.to(f32) / 4294967296.0
            gauss = u if gauss is None else gauss + u
        gauss = gauss - 6.0
        gray = (90.0 + 20.0 * gauss).round().clamp(1, 255)
        shell_val = (200.0 + 40.0 * _noise_fixed(xs, ys, zs, 4.0, seed, 8)).round().clamp(1, 255)
        v = torch.where(inner & (u1 < 0.2), gray, torch.zeros((), device=dev, dtype=f32))
        v = torch.where(shell, shell_val, v)
        g8 = v.to(torch.uint8)
        blk = torch.stack([g8, g8, g8, torch.full_like(g8, 255)], dim=-1)
        out[z0:z1] = blk.cpu().numpy()
    return out


def _noise_fixed(xs, ys, zs, cell: float, seed: int, salt: int) -> torch.Tensor:
    """Value noise whose lattice is anchored at the origin of the volume."""
    dev = xs.device
    gx, gy, gz = xs / cell, ys / cell, zs / cell
    ix, iy, iz = torch.floor(gx), torch.floor(gy), torch.floor(gz)
    fx, fy, fz = gx - ix, gy - iy, gz - iz
    fx, fy, fz = fx * fx * (3 - 2 * fx), fy * fy * (3 - 2 * fy), fz * fz * (3 - 2 * fz)
    ix, iy, iz = ix.to(torch.int64), iy.to(torch.int64), iz.to(torch.int64)
    lz = torch.arange(int(iz.min()), int(iz.max()) + 2, device=dev, dtype=torch.int64)
    ly = torch.arange(0, int(iy.max()) + 2, device=dev, dtype=torch.int64)
    lx = torch.arange(0, int(ix.max()) + 2, device=dev, dtype=torch.int64)
    lat = (_uniform(lx[None, None, :], ly[None, :, None], lz[:, None, None], seed, salt) * 2 - 1).to(torch.float32)
    iz = iz - int(lz[0])
    out = None
    for dz in (0, 1):
        wz = (fz if dz else 1 - fz)[:, None, None]
        for dy in (0, 1):
            wy = (fy if dy else 1 - fy)[None, :, None]
            for dx in (0, 1):
                wx = (fx if dx else 1 - fx)[None, None, :]
                v = lat[(iz + dz)[:, None, None], (iy + dy)[None, :, None], (ix + dx)[None, None, :]]
                term = v * (wz * wy * wx)
                out = term if out is None else out + term
    return out


def fire_ramp() -> np.ndarray:
    """256-entry black -> red -> yellow -> white colour ramp (uint8, (256, 3))."""
    t = np.arange(256) / 255.0
    r = np.clip(3 * t, 0, 1)
    g = np.clip(3 * t - 1, 0, 1)
    b = np.clip(3 * t - 2, 0, 1)
    return np.round(np.stack([r, g, b], 1) * 255).astype(np.uint8)


def gas_field(n: int = 1024, seed: int = 2, slope: float = -2.5, zero_percentile: float = 60.0,
              device=None, as_tensor: bool = False):
    """Cosmology-like gas density (the TNG volume stand-in), n^3 RGBA8.

    A Gaussian random field with power spectrum P(k) ~ k^slope, exponentiated
    to a log-normal density, log10-mapped onto the 256-entry fire ramp; voxels
    below the given percentile of the density are zeroed.  With as_tensor the
    result stays on `device` as a torch uint8 tensor (n, n, n, 4)."""
    dev = _device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    kz = torch.fft.fftfreq(n, device=dev)
    kx = torch.fft.rfftfreq(n, device=dev)
    noise = torch.randn((n, n, n), generator=gen, device=dev, dtype=torch.float32)
    spec = torch.fft.rfftn(noise)
    del noise
    for z0 in range(0, n, 64):  # scale by sqrt(P(k)) slab by slab to bound temporaries
        z1 = min(n, z0 + 64)
        k2 = kz[z0:z1, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2
        amp = torch.where(k2 > 0, k2.clamp_min(1e-12) ** (slope / 4.0), torch.zeros_like(k2))
        spec[z0:z1] *= amp
    field = torch.fft.irfftn(spec, s=(n, n, n))
    del spec
    field = (field - field.mean()) / field.std()
    # log10 of the log-normal density exp(field) is field / ln 10
    logd = field / math.log(10.0)
    del field
    flat = logd.reshape(-1)
    idx = torch.randint(0, flat.numel(), (1 << 22,), generator=gen, device=dev)
    sample = flat[idx]
    cut = torch.quantile(sample, zero_percentile / 100.0)
    lo, hi = torch.quantile(sample, 0.001), torch.quantile(sample, 0.999)
    ramp = torch.from_numpy(fire_ramp()).to(dev)
    out = torch.empty((n, n, n, 4), dtype=torch.uint8, device=dev) if as_tensor else np.empty((n, n, n, 4), np.uint8)
    for z0 in range(0, n, 64):
        z1 = min(n, z0 + 64)
        d = logd[z0:z1]
        i = ((d - lo) / (hi - lo) * 255).clamp(0, 255).round().to(torch.int64)
        rgb = ramp[i]
        rgb[d < cut] = 0
        blk = torch.cat([rgb, torch.full(rgb.shape[:-1] + (1,), 255, dtype=torch.uint8, device=dev)], dim=-1)
        if as_tensor:
            out[z0:z1] = blk
        else:
            out[z0:z1] = blk.cpu().numpy()
    return out


def random_grid(dz: int, dy: int, dx: int, seed: int = 0, density: float = 0.3, levels: int = 256) -> np.ndarray:
    """Small random test grid: `density` of voxels non-zero, alpha 255."""
    rng = np.random.default_rng(seed)
    g = np.zeros((dz, dy, dx, 4), np.uint8)
    m = rng.random((dz, dy, dx)) < density
    vals = rng.integers(0, levels, (int(m.sum()), 3)) * (255 // max(1, levels - 1))
    g[m, :3] = np.minimum(vals, 255).astype(np.uint8)
    g[..., 3] = 255
    return g
