"""Seeded synthetic float32 fields with the shapes and value distributions of the
workloads FZ-GPU is measured on (CESM CLDHGH 3600x1800, EXAFEL 39200x388, Hurricane
CLOUDf48 500x500x100, README.md:28-37).  The real SDRBench files are not available
offline; these generators stand in for them.  Fields are returned as flat float32
arrays in x-fastest order.
"""
from __future__ import annotations

import math

import numpy as np


def _plane_waves_2d(x, y, rng, terms, lam_lo, lam_hi):
    xs = np.arange(x, dtype=np.float64)
    ys = np.arange(y, dtype=np.float64)
    f = np.zeros((y, x), np.float64)
    for _ in range(terms):
        lam = math.exp(rng.uniform(math.log(lam_lo), math.log(lam_hi)))
        th = rng.uniform(0, 2 * math.pi)
        ph = rng.uniform(0, 2 * math.pi)
        amp = rng.uniform(0.2, 1.0)
        kx, ky = 2 * math.pi * math.cos(th) / lam, 2 * math.pi * math.sin(th) / lam
        u = kx * xs
        v = ky * ys + ph
        # sin(u + v) = sin u cos v + cos u sin v, evaluated as two outer products
        f += amp * (np.outer(np.cos(v), np.sin(u)) + np.outer(np.sin(v), np.cos(u)))
    return f


def smooth2d(x, y, seed=0, zero_frac=0.30, noise=1e-4):
    """cesm-like 3600x1800 field: 16 random 2D sinusoids (wavelength 50-1000 cells) normalised to
    [0,1], ~30% exact zeros in contiguous patches (thresholded low-frequency mask),
    N(0, 1e-4) noise, clipped at 0."""
    rng = np.random.default_rng(seed)
    f = _plane_waves_2d(x, y, rng, 16, 50.0, 1000.0)
    f = (f - f.min()) / max(f.max() - f.min(), 1e-30)
    mask_field = _plane_waves_2d(x, y, rng, 4, 400.0, 2000.0)
    thr = np.quantile(mask_field[:: max(1, y // 64), :: max(1, x // 64)], zero_frac)
    f += rng.normal(0.0, noise, size=f.shape)
    f[mask_field < thr] = 0.0
    np.maximum(f, 0.0, out=f)
    return f.astype(np.float32).ravel()


def peaks2d(x, y, seed=1, npeaks=None):
    """exafel-like 39200x388 field: Gaussian(0, 0.5) background plus ~2000 seeded 2D Gaussian peaks
    (sigma 1-3 px, amplitude log-uniform 10-1e4), a heavy-tailed value range."""
    rng = np.random.default_rng(seed)
    f = rng.normal(0.0, 0.5, size=(y, x)).astype(np.float32)
    if npeaks is None:
        npeaks = max(1, int(round(2000 * (x * y) / (39200 * 388))))
    for _ in range(npeaks):
        cx, cy = rng.uniform(0, x), rng.uniform(0, y)
        sg = rng.uniform(1.0, 3.0)
        amp = math.exp(rng.uniform(math.log(10.0), math.log(1e4)))
        r = int(math.ceil(4 * sg))
        x0, x1 = max(0, int(cx) - r), min(x, int(cx) + r + 1)
        y0, y1 = max(0, int(cy) - r), min(y, int(cy) + r + 1)
        if x0 >= x1 or y0 >= y1:
            continue
        gx = np.exp(-0.5 * ((np.arange(x0, x1) - cx) / sg) ** 2)
        gy = np.exp(-0.5 * ((np.arange(y0, y1) - cy) / sg) ** 2)
        f[y0:y1, x0:x1] += (amp * np.outer(gy, gx)).astype(np.float32)
    return f.ravel()


def smooth3d(x, y, z, seed=2, zero_frac=0.40):
    """hurricane-like 500x500x100 field: 32 random 3D sinusoids plus a seeded vortex-like radial profile,
    ~40% of voxels exactly 0 (values below the 40th percentile are cut to 0)."""
    rng = np.random.default_rng(seed)
    xs = np.arange(x, dtype=np.float32)
    ys = np.arange(y, dtype=np.float32)
    zs = np.arange(z, dtype=np.float32)
    f = np.zeros((z, y, x), np.float32)
    for _ in range(32):
        lams = np.exp(rng.uniform(math.log(20.0), math.log(400.0), size=3))
        ph = rng.uniform(0, 2 * math.pi, size=3)
        amp = np.float32(rng.uniform(0.2, 1.0))
        sx = np.sin(2 * np.pi * xs / lams[0] + ph[0]).astype(np.float32)
        sy = np.sin(2 * np.pi * ys / lams[1] + ph[1]).astype(np.float32)
        sz = np.sin(2 * np.pi * zs / lams[2] + ph[2]).astype(np.float32)
        f += amp * sz[:, None, None] * (sy[:, None] * sx[None, :])[None, :, :]
    # vortex: a radial profile around a seeded axis parallel to z
    cx, cy = rng.uniform(0.3, 0.7) * x, rng.uniform(0.3, 0.7) * y
    rr = np.sqrt((xs[None, :] - cx) ** 2 + (ys[:, None] - cy) ** 2)
    core = max(x, y) / 8.0
    prof = (4.0 * (rr / core) * np.exp(1.0 - rr / core)).astype(np.float32)
    f += prof[None, :, :]
    sub = f[:: max(1, z // 16), :: max(1, y // 32), :: max(1, x // 32)]
    thr = np.float32(np.quantile(sub, zero_frac))
    f -= thr
    np.maximum(f, 0.0, out=f)
    return f.ravel()


def smooth1d(n, seed=5):
    """A 1D smooth series (random-walk of a low-pass signal) with a few zero runs."""
    rng = np.random.default_rng(seed)
    t = np.arange(n, dtype=np.float64)
    f = np.zeros(n, np.float64)
    for _ in range(8):
        lam = math.exp(rng.uniform(math.log(30.0), math.log(5000.0)))
        f += rng.uniform(0.2, 1.0) * np.sin(2 * math.pi * t / lam + rng.uniform(0, 6.3))
    f += np.cumsum(rng.normal(0, 0.01, n))
    f = (f - f.min()) / max(f.max() - f.min(), 1e-30)
    f[f < 0.1] = 0.0
    return f.astype(np.float32)


def field(kind, dims, seed):
    """Dispatch by kind: 'smooth2d', 'peaks2d', 'smooth3d', 'smooth1d'."""
    x, y, z = dims
    if kind == "smooth2d":
        return smooth2d(x, y, seed)
    if kind == "peaks2d":
        return peaks2d(x, y, seed)
    if kind == "smooth3d":
        return smooth3d(x, y, z, seed)
    if kind == "smooth1d":
        return smooth1d(x * y * z, seed)
    raise ValueError(kind)


# The three single-field workloads: (name, kind, dims, seed, relative error bounds)
CONFIGS = [
    ("cesm-like 3600x1800", "smooth2d", (3600, 1800, 1), 0, (1e-3,)),
    ("exafel-like 39200x388", "peaks2d", (39200, 388, 1), 1, (1e-3, 1e-4)),
    ("hurricane-like 500x500x100", "smooth3d", (500, 500, 100), 2, (1e-2, 1e-3, 1e-4)),
]


# ------------------------------------------------------------------ mixed batches
def _dims_for(n, nd, rng):
    """Dims with x*y*z <= n close to n for a 1D/2D/3D field of about n elements."""
    if nd == 1:
        return (n, 1, 1)
    if nd == 2:
        x = max(2, int(round(math.sqrt(n * rng.uniform(0.5, 4.0)))))
        return (x, max(2, n // x), 1)
    s = max(2, int(round(n ** (1 / 3))))
    return (s, s, max(2, n // (s * s)))


def mixed_specs(count, seed=3, lo_bytes=64 << 10, hi_bytes=256 << 20, ebs=(1e-2, 1e-3, 1e-4)):
    """The mixed batch and the request trace: `count` fields with sizes log-uniform between 64 KB and 256 MB,
    mixed 1D/2D/3D, each with an eb drawn from {1e-2, 1e-3, 1e-4}.  Returns
    [(kind, dims, eb, seed)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        nbytes = math.exp(rng.uniform(math.log(lo_bytes), math.log(hi_bytes)))
        n = max(64, int(nbytes // 4))
        nd = int(rng.integers(1, 4))
        dims = _dims_for(n, nd, rng)
        kind = {1: "smooth1d", 2: "smooth2d" if rng.random() < 0.6 else "peaks2d", 3: "smooth3d"}[nd]
        out.append((kind, dims, float(ebs[int(rng.integers(0, len(ebs)))]), seed * 100000 + i))
    return out


def field_torch(kind, dims, seed, device="cuda"):
    """Device-side generator of the same field families (sums of separable sinusoids with
    zero patches, or Gaussian peaks on a noisy background), for multi-GB batches.  It
    is not bit-identical to the numpy generators, only alike in distribution."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    x, y, z = dims
    f32 = torch.float32

    def U(*shape, lo=0.0, hi=1.0):
        return lo + (hi - lo) * torch.rand(*shape, generator=g, device=device, dtype=f32)

    if kind == "smooth1d":
        t = torch.arange(x * y * z, device=device, dtype=f32)
        f = torch.zeros_like(t)
        for _ in range(6):
            lam = torch.exp(U(1, lo=math.log(30.0), hi=math.log(5000.0)))
            f += U(1, lo=0.2) * torch.sin(2 * math.pi * t / lam + U(1, hi=6.28))
        f = (f - f.min()) / (f.max() - f.min() + 1e-30)
        f[f < 0.1] = 0
        return f
    if kind == "peaks2d":
        f = 0.5 * torch.randn(y, x, generator=g, device=device, dtype=f32)
        npk = max(1, int(2000 * x * y / (39200 * 388)))
        cx, cy = U(npk, hi=float(x)), U(npk, hi=float(y))
        amp = torch.exp(U(npk, lo=math.log(10.0), hi=math.log(1e4)))
        ix = cx.long().clamp(0, x - 1)
        iy = cy.long().clamp(0, y - 1)
        f[iy, ix] += amp  # point sources, then a 3x3 blur gives sigma ~1 px peaks
        f = torch.nn.functional.avg_pool2d(f[None, None], 3, 1, 1)[0, 0] * 9 / 4
        return f.reshape(-1).contiguous()
    # smooth2d / smooth3d: separable products of sinusoids
    zs = torch.arange(z, device=device, dtype=f32)[:, None, None]
    ys = torch.arange(y, device=device, dtype=f32)[None, :, None]
    xs = torch.arange(x, device=device, dtype=f32)[None, None, :]
    f = torch.zeros(z, y, x, device=device, dtype=f32)
    for _ in range(8):
        lx, ly, lz = torch.exp(U(3, lo=math.log(20.0), hi=math.log(800.0)))
        ph = U(3, hi=6.28)
        term = torch.sin(2 * math.pi * xs / lx + ph[0]) * torch.sin(2 * math.pi * ys / ly + ph[1])
        if z > 1:
            term = term * torch.sin(2 * math.pi * zs / lz + ph[2])
        f += U(1, lo=0.2) * term
    thr = torch.quantile(f.reshape(-1)[:: max(1, f.numel() // 65536)], 0.35)
    f = torch.clamp(f - thr, min=0)
    return f.reshape(-1).contiguous()
