"""Seeded synthetic multiview data (beads + ellipsoid, rotated PSFs, Poisson noise).

The reference measures on local microscopy datasets that are not distributed with it;
this generator stands in for them with the shapes, sizes and value distributions of
the named workloads:

* object: random Gaussian beads (centre U[0, dim), sigma U[s0, s1], amplitude
  U[100, 1000]) plus a smooth ellipsoid of intensity 50 (semi-axes 0.35 * dim, edge
  smoothed with sigma 2);
* PSFs: anisotropic Gaussians (optionally with two axial side lobes at +-2.5 sigma_z,
  amplitude 0.1), rotated about y with trilinear resampling in the same box, clamped
  at 0 and sum-normalised;
* images: object convolved with each view's PSF in float64, background 10 added,
  Poisson sampled, clamped to >= 1 inside the volume (the reference's minValueImg,
  MultiViewDeconvolution.java:49);
* weights: all 1, or a cosine blend per view (1 in the centre, cosine fall-off over
  12 voxels to the view's edge along its rotated x axis).

Arrays are float32 ``[z][y][x]``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

try:
    import scipy.fft as _fft

    def _rfftn(a, s=None):
        return _fft.rfftn(a, s=s, workers=-1)

    def _irfftn(a, s):
        return _fft.irfftn(a, s=s, workers=-1)
except Exception:  # pragma: no cover
    def _rfftn(a, s=None):
        return np.fft.rfftn(a, s=s)

    def _irfftn(a, s):
        return np.fft.irfftn(a, s=s)


def _gauss_box(size_xyz, sig_xyz, side_lobes=False):
    sx, sy, sz = size_xyz
    z, y, x = np.meshgrid(np.arange(sz) - sz // 2, np.arange(sy) - sy // 2,
                          np.arange(sx) - sx // 2, indexing="ij")
    g = np.exp(-0.5 * ((x / sig_xyz[0]) ** 2 + (y / sig_xyz[1]) ** 2 + (z / sig_xyz[2]) ** 2))
    if side_lobes:
        for s in (-1.0, 1.0):
            dz = z - s * 2.5 * sig_xyz[2]
            g = g + 0.1 * np.exp(-0.5 * ((x / sig_xyz[0]) ** 2 + (y / sig_xyz[1]) ** 2 +
                                         (dz / sig_xyz[2]) ** 2))
    return g


def _trilinear(vol, zc, yc, xc):
    """Sample vol (zero outside) at fractional coordinates."""
    nz, ny, nx = vol.shape
    z0 = np.floor(zc).astype(np.int64)
    y0 = np.floor(yc).astype(np.int64)
    x0 = np.floor(xc).astype(np.int64)
    fz, fy, fx = zc - z0, yc - y0, xc - x0
    out = np.zeros(zc.shape, dtype=np.float64)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                zi, yi, xi = z0 + dz, y0 + dy, x0 + dx
                ok = (zi >= 0) & (zi < nz) & (yi >= 0) & (yi < ny) & (xi >= 0) & (xi < nx)
                wgt = (fz if dz else 1 - fz) * (fy if dy else 1 - fy) * (fx if dx else 1 - fx)
                v = np.zeros(zc.shape)
                v[ok] = vol[zi[ok], yi[ok], xi[ok]]
                out += wgt * v
    return out


def make_psf(size_xyz, sigma_xy, sigma_z, angle_deg, side_lobes=False):
    """Gaussian (+ optional side lobes) PSF rotated about y by angle_deg in its own
    box (odd sizes), clamped >= 0 and sum-normalised; float32 [z][y][x]."""
    base = _gauss_box(size_xyz, (sigma_xy, sigma_xy, sigma_z), side_lobes)
    sx, sy, sz = size_xyz
    z, y, x = np.meshgrid(np.arange(sz) - sz // 2, np.arange(sy) - sy // 2,
                          np.arange(sx) - sx // 2, indexing="ij")
    a = math.radians(angle_deg)
    # inverse rotation about y: sample the unrotated PSF at R^-1 p
    xr = math.cos(a) * x - math.sin(a) * z
    zr = math.sin(a) * x + math.cos(a) * z
    rot = _trilinear(base, zr + sz // 2, y + sy // 2, xr + sx // 2)
    rot = np.maximum(rot, 0)
    rot /= rot.sum()
    return rot.astype(np.float32)


def make_object(dims_xyz, n_beads, rng, sigma=(1.0, 2.0), ellipsoid=50.0):
    nx, ny, nz = dims_xyz
    obj = np.zeros((nz, ny, nx), dtype=np.float64)
    if ellipsoid:
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        r = np.sqrt(((x - (nx - 1) / 2) / (0.35 * nx)) ** 2 + ((y - (ny - 1) / 2) / (0.35 * ny)) ** 2 +
                    ((z - (nz - 1) / 2) / (0.35 * nz)) ** 2)
        # signed distance (in voxels, approx.) to the ellipsoid surface, smoothed edge sigma 2
        dist = (r - 1.0) * (0.35 * min(dims_xyz))
        obj += ellipsoid * 0.5 * (1.0 - np.tanh(dist / (2.0 * math.sqrt(2.0))))
    cx = rng.uniform(0, nx, n_beads)
    cy = rng.uniform(0, ny, n_beads)
    cz = rng.uniform(0, nz, n_beads)
    sg = rng.uniform(sigma[0], sigma[1], n_beads)
    amp = rng.uniform(100, 1000, n_beads)
    for i in range(n_beads):
        r = int(math.ceil(4 * sg[i]))
        x0, x1 = max(0, int(cx[i]) - r), min(nx, int(cx[i]) + r + 1)
        y0, y1 = max(0, int(cy[i]) - r), min(ny, int(cy[i]) + r + 1)
        z0, z1 = max(0, int(cz[i]) - r), min(nz, int(cz[i]) + r + 1)
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        zz, yy, xx = np.meshgrid(np.arange(z0, z1), np.arange(y0, y1), np.arange(x0, x1), indexing="ij")
        d2 = (xx - cx[i]) ** 2 + (yy - cy[i]) ** 2 + (zz - cz[i]) ** 2
        obj[z0:z1, y0:y1, x0:x1] += amp[i] * np.exp(-0.5 * d2 / sg[i] ** 2)
    return obj


def blur(obj, psf):
    """Linear convolution (zero outside) of obj with a centred psf, float64."""
    s = [obj.shape[d] + psf.shape[d] - 1 for d in range(3)]
    f = _irfftn(_rfftn(obj, s) * _rfftn(psf.astype(np.float64), s), s)
    c = [psf.shape[d] // 2 for d in range(3)]
    return f[c[0]:c[0] + obj.shape[0], c[1]:c[1] + obj.shape[1], c[2]:c[2] + obj.shape[2]]


def cosine_weight(dims_xyz, angle_deg, blend=12.0):
    nx, ny, nz = dims_xyz
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    a = math.radians(angle_deg)
    u = (x - (nx - 1) / 2) * math.cos(a) + (z - (nz - 1) / 2) * math.sin(a)
    half = 0.5 * (abs(nx * math.cos(a)) + abs(nz * math.sin(a)))
    d = half - np.abs(u)  # distance to the view's edge along its rotated x axis
    w = np.where(d >= blend, 1.0, 0.5 * (1 - np.cos(np.pi * np.clip(d, 0, blend) / blend)))
    return w.astype(np.float32)


@dataclass
class MultiviewData:
    images: list
    weights: list
    psfs: list
    obj: np.ndarray


def make_dataset(dims_xyz, angles, psf_size_xyz, n_beads=200, seed=1001, sigma_xy=1.5, sigma_z=4.5,
                 side_lobes=False, weights="ones", background=10.0, bead_sigma=(1.0, 2.0)):
    """psf_size_xyz: one size for every view, or a list with one size per view."""
    rng = np.random.Generator(np.random.PCG64(seed))
    obj = make_object(dims_xyz, n_beads, rng, sigma=bead_sigma)
    sizes = psf_size_xyz if isinstance(psf_size_xyz[0], (tuple, list)) else [psf_size_xyz] * len(angles)
    psfs = [make_psf(sz, sigma_xy, sigma_z, a, side_lobes) for sz, a in zip(sizes, angles)]
    imgs, ws = [], []
    for a, p in zip(angles, psfs):
        b = blur(obj, p) + background
        b = rng.poisson(np.maximum(b, 0)).astype(np.float32)
        imgs.append(np.maximum(b, 1.0).astype(np.float32))
        if weights == "ones":
            ws.append(np.ones(obj.shape, dtype=np.float32))
        else:
            ws.append(cosine_weight(dims_xyz, a))
    return MultiviewData(images=imgs, weights=ws, psfs=psfs, obj=obj.astype(np.float32))


def config_small(seed=1001):
    """2 views, 128x128x64, PSF 15x15x31 at 0/90 degrees, all-one weights."""
    return make_dataset((128, 128, 64), (0.0, 90.0), (15, 15, 31), n_beads=200, seed=seed)


def config_256(seed=1002):
    """4 views, 256^3, 31x31x61 Gaussian-plus-side-lobe PSFs at 0/45/90/135 degrees,
    cosine-blended weights (raw; normalise with the reference's hard rule)."""
    return make_dataset((256, 256, 256), (0.0, 45.0, 90.0, 135.0), (31, 31, 61), n_beads=200,
                        seed=seed, side_lobes=True, weights="cosine")


# per-view PSF sizes of the 6-view workload: 21 ... 41 voxels in x/y, 41 ... 81 in z
PSF_SIZES_6 = [(21, 21, 41), (25, 25, 49), (29, 29, 57), (33, 33, 65), (37, 37, 73), (41, 41, 81)]


def config_512(seed=1003):
    """6 views, 512 x 512 x 256, Gaussian-plus-side-lobe PSFs of different sizes per view
    (21-41 voxels in x/y, 41-81 in z) at 0/30/.../150 degrees, cosine-blended weights."""
    return make_dataset((512, 512, 256), (0.0, 30.0, 60.0, 90.0, 120.0, 150.0), PSF_SIZES_6, n_beads=800,
                        seed=seed, side_lobes=True, weights="cosine")


def config_large(device=0, seed=1005, dims_xyz=(1024, 1024, 512), n_views=8, n_objects=20000,
                 psf_size_xyz=(41, 41, 81)):
    """The large-volume stress case: 8 views of 1024 x 1024 x 512 recorded as uint16 and
    converted to float32, dense nuclei-like blobs (sigma U[3, 6], amplitude U[100, 1000]),
    Gaussian-plus-side-lobe PSFs 41 x 41 x 81 rotated in 45 degree steps, background 10,
    Poisson noise, cosine-blended weights.  Synthesised on the GPU with torch (at this size
    the host generator above would take minutes per view); returns images and weights as
    device tensors [z][y][x] and the PSFs as host arrays."""
    import torch

    dev = device if isinstance(device, str) else f"cuda:{device}"
    nx, ny, nz = dims_xyz
    rng = np.random.Generator(np.random.PCG64(seed))
    cx, cy, cz = rng.uniform(0, nx, n_objects), rng.uniform(0, ny, n_objects), rng.uniform(0, nz, n_objects)
    sg = rng.uniform(3.0, 6.0, n_objects)
    amp = rng.uniform(100, 1000, n_objects)
    # blobs in four sigma classes: amplitudes scattered at their centres, blurred by the
    # class's Gaussian in Fourier space (periodic; the objects keep 3 sigma from the border)
    fz = torch.fft.fftfreq(nz, device=dev).view(-1, 1, 1)
    fy = torch.fft.fftfreq(ny, device=dev).view(1, -1, 1)
    fx = torch.fft.rfftfreq(nx, device=dev).view(1, 1, -1)
    f2 = fz * fz + fy * fy + fx * fx
    obj = torch.zeros((nz, ny, nx), dtype=torch.float32, device=dev)
    edges = np.linspace(3.0, 6.0, 5)
    for c in range(4):
        sel = (sg >= edges[c]) & (sg <= edges[c + 1] if c == 3 else sg < edges[c + 1])
        s = float(0.5 * (edges[c] + edges[c + 1]))
        m = 3 * s
        ix = np.clip(cx[sel], m, nx - 1 - m).astype(np.int64)
        iy = np.clip(cy[sel], m, ny - 1 - m).astype(np.int64)
        iz = np.clip(cz[sel], m, nz - 1 - m).astype(np.int64)
        # peak amplitude a: a Gaussian of volume a (2 pi s^2)^(3/2)
        a = torch.from_numpy(amp[sel] * (2 * math.pi * s * s) ** 1.5).to(dev, torch.float32)
        spikes = torch.zeros_like(obj)
        flat = torch.from_numpy((iz * ny + iy) * nx + ix).to(dev)
        spikes.view(-1).index_add_(0, flat, a)
        spec = torch.fft.rfftn(spikes) * torch.exp(-2 * math.pi ** 2 * s * s * f2)
        obj += torch.fft.irfftn(spec, s=(nz, ny, nx))
        del spikes, spec
    obj.clamp_(min=0)
    angles = [45.0 * v for v in range(n_views)]
    psfs = [make_psf(psf_size_xyz, 1.5, 4.5, a, side_lobes=True) for a in angles]
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    imgs, ws = [], []
    pad = [obj.shape[d] + psfs[0].shape[d] - 1 for d in range(3)]
    ospec = torch.fft.rfftn(obj, s=pad)
    for a, p in zip(angles, psfs):
        pk = torch.from_numpy(p.astype(np.float32)).to(dev)
        b = torch.fft.irfftn(ospec * torch.fft.rfftn(pk, s=pad), s=pad)
        c = [p.shape[d] // 2 for d in range(3)]
        b = b[c[0]:c[0] + nz, c[1]:c[1] + ny, c[2]:c[2] + nx] + 10.0
        counts = torch.poisson(b.clamp(min=0), generator=gen).clamp_(1, 65535).to(torch.int32)
        del b
        img_u16 = counts.to(torch.int16)  # the recorded uint16 values (bit pattern)
        del counts
        imgs.append((img_u16.to(torch.int32) & 0xFFFF).to(torch.float32))  # uint16 -> float32
        del img_u16
        ws.append(_cosine_weight_torch(dims_xyz, a, dev))
    del ospec, obj
    return MultiviewData(images=imgs, weights=ws, psfs=psfs, obj=None)


def _cosine_weight_torch(dims_xyz, angle_deg, dev, blend=12.0):
    """cosine_weight on the GPU (the weight depends on x and z only)."""
    import torch

    nx, ny, nz = dims_xyz
    a = math.radians(angle_deg)
    x = torch.arange(nx, device=dev, dtype=torch.float64).view(1, -1)
    z = torch.arange(nz, device=dev, dtype=torch.float64).view(-1, 1)
    u = (x - (nx - 1) / 2) * math.cos(a) + (z - (nz - 1) / 2) * math.sin(a)
    half = 0.5 * (abs(nx * math.cos(a)) + abs(nz * math.sin(a)))
    d = half - u.abs()
    w = torch.where(d >= blend, torch.ones_like(d), 0.5 * (1 - torch.cos(math.pi * d.clamp(0, blend) / blend)))
    return w.to(torch.float32).view(nz, 1, nx).expand(nz, ny, nx).contiguous()
