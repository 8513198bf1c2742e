"""ctypes front end of the CPU oracle (oracle/mvr_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` -- as the checker and
the timed CPU restatement, never by the product library.

Every function mirrors a reference routine (cited in mvr_oracle.c); arrays are
numpy, C-contiguous ``[z][y][x]`` (x fastest), shapes passed as ``(x, y, z)`` sizes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "mvr_oracle.c")
_LIB = os.path.join(_HERE, "liboracle.so")

PSF_OPTIMIZATION_II, PSF_OPTIMIZATION_I, PSF_EFFICIENT_BAYESIAN, PSF_INDEPENDENT = 0, 1, 2, 3
EXT_ZERO, EXT_MIRROR_SINGLE, EXT_VALUE = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (OpenMP, no FMA contraction)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["gcc", "-O2", "-std=gnu11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", _LIB, _SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        P = C.c_void_p
        L.orc_fft1d.argtypes = [P, C.c_int, C.c_int]
        L.orc_mirror_single.argtypes = [C.c_long, C.c_long]
        L.orc_mirror_single.restype = C.c_long
        L.orc_convolve.argtypes = [P, P, C.c_int, C.c_double, P, P, P]
        L.orc_block_seq.argtypes = [P, P, P, P, P, P, P, P, P, C.c_double, C.c_float, C.c_float,
                                    C.c_int, P]
        L.orc_block_mul.argtypes = [P, P, C.c_int, P, P, P, P, P, P, P, C.c_double, C.c_float, P,
                                    C.c_int, P]
        L.orc_norm_to_sum1.argtypes = [P, C.c_long, C.c_int]
        L.orc_invert_kernel.argtypes = [P, P, P]
        L.orc_psf_init.argtypes = [C.c_int, P, P, C.c_int, C.c_int, P]
        L.orc_divide_into_blocks.argtypes = [P, P, P, P, C.c_int]
        L.orc_divide_into_blocks.restype = C.c_int
        L.orc_sort_blocks.argtypes = [P, C.c_int]
        L.orc_sort_blocks.restype = C.c_int
        L.orc_normalize_weights.argtypes = [C.c_int, P, C.c_long, C.c_double, C.c_int, C.c_float,
                                            C.c_float, P]
        L.orc_psi_init_avg.argtypes = [C.c_int, P, C.c_long, P, P]
        L.orc_psi_init_avg.restype = C.c_double
        L.orc_decon_run.argtypes = [C.c_int, P, P, P, P, P, P, P, P, C.c_int, C.c_int, C.c_double,
                                    C.c_float, P, C.c_int, C.c_int, P, P, P]
        L.orc_decon_run.restype = C.c_int
        L.orc_num_threads.restype = C.c_int
        L.orc_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _dims(a):
    """(x, y, z) sizes of a [z][y][x] array."""
    return np.array([a.shape[2], a.shape[1], a.shape[0]], dtype=np.int32)


def _ptr_array(arrs):
    return (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


def fft1d(x: np.ndarray, inverse: bool = False) -> np.ndarray:
    d = np.empty(2 * len(x), dtype=np.float64)
    d[0::2] = x.real
    d[1::2] = x.imag
    lib().orc_fft1d(_p(d), len(x), int(inverse))
    return d[0::2] + 1j * d[1::2]


def mirror_single(i: int, n: int) -> int:
    return lib().orc_mirror_single(i, n)


def convolve(block: np.ndarray, kernel: np.ndarray, ext: int, ext_value: float = 0.0) -> np.ndarray:
    block = np.ascontiguousarray(block, dtype=np.float32)
    kernel = np.ascontiguousarray(kernel, dtype=np.float32)
    out = np.empty(block.shape, dtype=np.float64)
    lib().orc_convolve(_p(block), _p(_dims(block)), ext, ext_value, _p(kernel), _p(_dims(kernel)),
                       _p(out))
    return out


def block_seq(psi, img, w, k1, k2, lam, min_value, max_intensity, fp64=False):
    """ComputeBlockSeqThreadCPU.runIteration on one block; returns (psi', (sum, max))."""
    img = np.ascontiguousarray(img, dtype=np.float32)
    w = np.ascontiguousarray(w, dtype=np.float32)
    k1 = np.ascontiguousarray(k1, dtype=np.float32)
    k2 = np.ascontiguousarray(k2, dtype=np.float32)
    st = np.zeros(2, dtype=np.float64)
    if fp64:
        p64 = np.array(psi, dtype=np.float64, order="C")
        lib().orc_block_seq(None, _p(p64), _p(img), _p(w), _p(_dims(img)), _p(k1), _p(_dims(k1)),
                            _p(k2), _p(_dims(k2)), lam, min_value, max_intensity, 1, _p(st))
        return p64, (st[0], st[1])
    p32 = np.array(psi, dtype=np.float32, order="C")
    lib().orc_block_seq(_p(p32), None, _p(img), _p(w), _p(_dims(img)), _p(k1), _p(_dims(k1)),
                        _p(k2), _p(_dims(k2)), lam, min_value, max_intensity, 0, _p(st))
    return p32, (st[0], st[1])


def block_mul(psi, imgs, ws, k1s, k2s, lam, min_value, max_intensities, fp64=False):
    """ComputeBlockMulThreadCPU.runIteration on one block; returns (psi', (sum, max))."""
    nv = len(imgs)
    imgs = [np.ascontiguousarray(a, dtype=np.float32) for a in imgs]
    ws = [np.ascontiguousarray(a, dtype=np.float32) for a in ws]
    k1s = [np.ascontiguousarray(a, dtype=np.float32) for a in k1s]
    k2s = [np.ascontiguousarray(a, dtype=np.float32) for a in k2s]
    k1d = np.concatenate([_dims(k) for k in k1s]).astype(np.int32)
    k2d = np.concatenate([_dims(k) for k in k2s]).astype(np.int32)
    mx = np.asarray(max_intensities, dtype=np.float32)
    st = np.zeros(2, dtype=np.float64)
    args = (nv, _ptr_array(imgs), _ptr_array(ws), _p(_dims(imgs[0])), _ptr_array(k1s), _p(k1d),
            _ptr_array(k2s), _p(k2d), lam, min_value, _p(mx))
    if fp64:
        p64 = np.array(psi, dtype=np.float64, order="C")
        lib().orc_block_mul(None, _p(p64), *args, 1, _p(st))
        return p64, (st[0], st[1])
    p32 = np.array(psi, dtype=np.float32, order="C")
    lib().orc_block_mul(_p(p32), None, *args, 0, _p(st))
    return p32, (st[0], st[1])


def norm_to_sum1(k: np.ndarray, T: int) -> np.ndarray:
    k = np.array(k, dtype=np.float32, order="C")
    lib().orc_norm_to_sum1(_p(k), k.size, T)
    return k


def invert_kernel(k: np.ndarray) -> np.ndarray:
    k = np.ascontiguousarray(k, dtype=np.float32)
    out = np.empty_like(k)
    lib().orc_invert_kernel(_p(k), _p(_dims(k)), _p(out))
    return out


def psf_init(kernels, psf_type: int, T: int):
    """DeconViewPSF.init for all views in order; returns (kernel1 list, kernel2 list)."""
    k1 = [np.array(k, dtype=np.float32, order="C") for k in kernels]
    k2 = [np.empty_like(k) for k in k1]
    kd = np.concatenate([_dims(k) for k in k1]).astype(np.int32)
    lib().orc_psf_init(len(k1), _ptr_array(k1), _p(kd), psf_type, T, _ptr_array(k2))
    return k1, k2


def divide_into_blocks(img_size, kernel2_size, block_size):
    """Blocks as dicts (offset, eff_offset, eff_size, eff_local), each (x, y, z)."""
    a = np.asarray(img_size, dtype=np.int64)
    k = np.asarray(kernel2_size, dtype=np.int64)
    b = np.asarray(block_size, dtype=np.int64)
    n = lib().orc_divide_into_blocks(_p(a), _p(k), _p(b), None, 0)
    if n < 0:
        return None
    out = np.zeros((n, 12), dtype=np.int64)
    lib().orc_divide_into_blocks(_p(a), _p(k), _p(b), _p(out), n)
    return [dict(offset=tuple(r[0:3]), eff_offset=tuple(r[3:6]), eff_size=tuple(r[6:9]),
                 eff_local=tuple(r[9:12])) for r in out]


def sort_dim(num_blocks, min_required: int = 1) -> int:
    nb = np.asarray(num_blocks, dtype=np.int64)
    return lib().orc_sort_blocks(_p(nb), min_required)


def normalize_weights(raw, osem=1.0, smooth=False, max_diff_range=0.1, scaling_range=0.05):
    raw = [np.ascontiguousarray(r, dtype=np.float32) for r in raw]
    out = [np.empty_like(r) for r in raw]
    lib().orc_normalize_weights(len(raw), _ptr_array(raw), raw[0].size, osem, int(smooth),
                                max_diff_range, scaling_range, _ptr_array(out))
    return out


def psi_init_avg(imgs):
    imgs = [np.ascontiguousarray(r, dtype=np.float32) for r in imgs]
    psi = np.empty_like(imgs[0])
    mx = np.zeros(len(imgs), dtype=np.float32)
    avg = lib().orc_psi_init_avg(len(imgs), _ptr_array(imgs), imgs[0].size, _p(psi), _p(mx))
    return psi, mx, avg


def gauss3_half_kernel(sigma: float) -> np.ndarray:
    """Gauss3.halfkernel of imglib2-algorithm (net.imglib2.algorithm.gauss3, the version
    pom-scijava 43.0.0 manages; not vendored in the reference): size max(2, (int)(3 sigma +
    0.5) + 1), h[0] = 1, h[x] = exp(-x^2 / (2 sigma^2)), normalised so that
    h[0] + 2 sum_{x>0} h[x] = 1."""
    hs = max(2, int(3.0 * sigma + 0.5) + 1)
    x = np.arange(hs, dtype=np.float64)
    h = np.exp(-(x * x) / (2.0 * sigma * sigma))
    h[0] = 1.0
    return h / (2.0 * (0.5 + h[1:].sum()))


def gauss3(vol: np.ndarray, sigma: float) -> np.ndarray:
    """Gauss3.gauss(sigma on every axis, Views.extendMirrorSingle(vol), vol): separable
    symmetric convolution along x, then y, then z, mirror-single extension, float64."""
    h = gauss3_half_kernel(sigma)
    hs = len(h)
    full = np.concatenate([h[:0:-1], h])
    out = np.asarray(vol, dtype=np.float64)
    for axis in (2, 1, 0):  # x, y, z of a [z][y][x] array
        n = out.shape[axis]
        idx = np.arange(-(hs - 1), n + hs - 1)
        if n > 1:
            p = 2 * n - 2
            idx = np.mod(idx, p)
            idx = np.where(idx >= n, p - idx, idx)
        else:
            idx = np.zeros_like(idx)
        ext = np.take(out, idx, axis=axis)
        acc = np.zeros_like(out)
        for k in range(2 * hs - 1):
            sl = [slice(None)] * 3
            sl[axis] = slice(k, k + n)
            acc += full[k] * ext[tuple(sl)]
        out = acc
    return out


def psi_init_blurred_fused(imgs, weights, sigma: float = 5.0):
    """PsiInitBlurredFused.runInitialization (deconvolution/init/PsiInitBlurredFused.java
    66-127) with FusedNonZeroRandomAccess.get (deconvolution/util/
    FusedNonZeroRandomAccess.java 63-102): psi = sum(I w) / sum(w) over the views with
    I > 0 (0 where the weights sum to 0), then Gauss3 with sigma; avg = the mean over voxels
    with data of the mean of those views; max = per-view maximum.  Returns (psi float32,
    max float32[views], avg)."""
    I = np.stack([np.asarray(a, dtype=np.float64) for a in imgs])
    Wt = np.stack([np.asarray(a, dtype=np.float64) for a in weights])
    pos = I > 0
    sumI = np.where(pos, I * Wt, 0.0).sum(0)
    sumW = np.where(pos, Wt, 0.0).sum(0)
    fused = np.where(sumW > 0, sumI / np.where(sumW > 0, sumW, 1.0), 0.0).astype(np.float32)
    cnt = pos.sum(0)
    tot = np.where(pos, I, 0.0).sum(0)
    has = cnt > 0
    avg = float((tot[has] / cnt[has]).sum() / has.sum()) if has.any() else float("nan")
    if np.isnan(avg):
        avg = 1.0
    mx = np.array([np.where(pos[v], I[v], 0.0).max() for v in range(len(imgs))], dtype=np.float32)
    return gauss3(fused, sigma).astype(np.float32), mx, avg


def psi_init_avg_approx(imgs):
    """PsiInitAvgApprox.runInitialization (deconvolution/init/PsiInitAvgApprox.java
    49-106) with PsiInitAvgApproxThread.call (57-84): per view the mean and maximum of the
    y-z slice at x = nx / 2; avg = mean of the views' slice means, psi = avg.  Returns
    (psi, max, avg)."""
    means, mx = [], []
    for a in imgs:
        sl = np.asarray(a, dtype=np.float64)[:, :, a.shape[2] // 2]
        means.append(sl.mean())
        mx.append(sl.max())
    avg = float(np.mean(means))
    if np.isnan(avg):
        avg = 1.0
    psi = np.full(imgs[0].shape, np.float32(avg), dtype=np.float32)
    return psi, np.array(mx, dtype=np.float32), avg


def decon_run(psi, imgs, ws, k1s, k2s, block_size, iters, mul=False, lam=0.0, min_value=1e-4,
              max_intensities=None, filter_blocks=True, fp64=False):
    """MultiViewDeconvolution{Seq,Mul}.runIterations with the reference's block order.

    Returns (psi, stats[n_steps, 2])."""
    nv = len(imgs)
    D = np.array([psi.shape[2], psi.shape[1], psi.shape[0]], dtype=np.int64)
    imgs = [np.ascontiguousarray(a, dtype=np.float32) for a in imgs]
    ws = [np.ascontiguousarray(a, dtype=np.float32) for a in ws]
    k1s = [np.ascontiguousarray(a, dtype=np.float32) for a in k1s]
    k2s = [np.ascontiguousarray(a, dtype=np.float32) for a in k2s]
    k1d = np.concatenate([_dims(k) for k in k1s]).astype(np.int32)
    k2d = np.concatenate([_dims(k) for k in k2s]).astype(np.int32)
    b = np.asarray(block_size, dtype=np.int32)
    mx = np.asarray(max_intensities, dtype=np.float32)
    nsteps = iters * (1 if mul else nv)
    st = np.zeros((nsteps, 2), dtype=np.float64)
    if fp64:
        p64 = np.array(psi, dtype=np.float64, order="C")
        p32 = None
    else:
        p32 = np.array(psi, dtype=np.float32, order="C")
        p64 = None
    rc = lib().orc_decon_run(nv, _p(D), _ptr_array(imgs), _ptr_array(ws), _ptr_array(k1s), _p(k1d),
                             _ptr_array(k2s), _p(k2d), _p(b), iters, int(mul), lam, min_value, _p(mx),
                             int(filter_blocks), int(fp64), _p(p32), _p(p64), _p(st))
    if rc != 0:
        raise ValueError("block size smaller than the doubled kernel")
    return (p64 if fp64 else p32), st


# ---- input preparation (ProcessInputImages.fuseGroups) ----------------------------------

def blending_lut():
    """BlendingRealRandomAccess's static table (fusion/transformed/weights/
    BlendingRealRandomAccess.java:38-47): d from 0 in steps of 0.001 accumulated in double,
    entry (int)(d * 1000 + 0.5) = (cos((1 - d) pi) + 1) / 2."""
    import math

    lut = np.zeros(1001)
    d = 0.0
    while d <= 1.0001:
        lut[int(d * 1000.0 + 0.5)] = (math.cos((1 - d) * math.pi) + 1) / 2
        d = d + 0.001
    return lut


def blending_weight(loc, dims_xyz, border, rng, lut=None):
    """BlendingRealRandomAccess.computeWeight (:96-125) on [0, dims - 1] at float32
    locations loc[..., 3] (x, y, z), float arithmetic, the table product in double."""
    lut = blending_lut() if lut is None else lut
    loc = np.asarray(loc, dtype=np.float32)
    w = np.ones(loc.shape[:-1], dtype=np.float32)
    zero = np.zeros(loc.shape[:-1], dtype=bool)
    tmps = []
    for d in range(3):
        l = loc[..., d]
        a = l - np.float32(border[d])
        b = (np.float32(dims_xyz[d] - 1) - l) - np.float32(border[d])
        t = np.minimum(a, b)
        zero |= t <= 0
        tmps.append(t)
    for d in range(3):
        rel = tmps[d] / np.float32(rng[d])
        use = rel < 1
        idx = np.clip((rel.astype(np.float64) * 1000.0 + 0.5).astype(np.int64), 0, 1000)
        w = np.where(use, (w.astype(np.float64) * lut[idx]).astype(np.float32), w)
    return np.where(zero, np.float32(0), w)


def _invert_affine(m):
    """Inverse of a 3 x 4 affine transform by the adjugate of its 3 x 3 part."""
    m = np.asarray(m, dtype=np.float64).reshape(3, 4)
    a, b, c, d = m[0, 0], m[0, 1], m[0, 2], m[0, 3]
    e, f, g, h = m[1, 0], m[1, 1], m[1, 2], m[1, 3]
    i, j, k, l = m[2, 0], m[2, 1], m[2, 2], m[2, 3]
    det = a * (f * k - g * j) - b * (e * k - g * i) + c * (e * j - f * i)
    r = 1.0 / det
    A = np.array([[(f * k - g * j) * r, (c * j - b * k) * r, (b * g - c * f) * r],
                  [(g * i - e * k) * r, (a * k - c * i) * r, (c * e - a * g) * r],
                  [(e * j - f * i) * r, (b * i - a * j) * r, (a * f - b * e) * r]])
    t = np.array([-(A[q, 0] * d + A[q, 1] * h + A[q, 2] * l) for q in range(3)])
    return np.concatenate([A, t.reshape(3, 1)], axis=1)


def apply_affine(m, s):
    """AffineTransform3D.apply (imglib2-realtransform) on s[..., 3] (x, y, z): each output
    coordinate s0 m0 + s1 m1 + s2 m2 + m3, summed left to right in double."""
    m = np.asarray(m, dtype=np.float64).reshape(3, 4)
    s = np.asarray(s, dtype=np.float64)
    return np.stack([((s[..., 0] * m[r, 0] + s[..., 1] * m[r, 1]) + s[..., 2] * m[r, 2]) + m[r, 3]
                     for r in range(3)], axis=-1)


_GRAY = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1))


def nlinear(get, t):
    """Linear interpolation as imglib2's NLinearInterpolator3D.get (imglib2 8.0.0, the
    interpolator of Views.interpolate with NLinearInterpolatorFactory): t[..., 3] double
    positions (x, y, z); get(ix, iy, iz) returns float32 values of the extended image.
    Weights in double (t - floor t, products x * y * z), each corner's value times its
    weight rounded to float, the corners summed in float in the Gray-code order 000, 100,
    110, 010, 011, 111, 101, 001."""
    t = np.asarray(t, dtype=np.float64)
    f = np.floor(t)
    w = t - f
    u = 1.0 - w
    fi = f.astype(np.int64)
    acc = None
    for dx, dy, dz in _GRAY:
        wgt = ((w[..., 0] if dx else u[..., 0]) * (w[..., 1] if dy else u[..., 1])) * (w[..., 2] if dz else u[..., 2])
        v = np.asarray(get(fi[..., 0] + dx, fi[..., 1] + dy, fi[..., 2] + dz), dtype=np.float32)
        term = (v.astype(np.float64) * wgt).astype(np.float32)
        acc = term if acc is None else (acc + term).astype(np.float32)
    return acc


def fuse_group(views, bb_min, bb_dims):
    """ProcessInputImages.fuseGroups (deconvolution/util/ProcessInputImages.java:279-399)
    for one group: each view (dict: img [z][y][x], model 3 x 4 view -> world, optional
    'fusion' / 'decon' = (border xyz, range xyz)) is transformed into the bounding box with
    linear interpolation, max(1, .) strictly inside the view and 0 outside
    (TransformedInputRandomAccess.get, AbstractTransformedIntervalRandomAccess
    .intersectsLinearInterpolation), weighted by its blending and averaged (FusedRandomAccess
    .get); the deconvolution weight is the sum of the views' deconvolution blendings
    (CombineWeightsSumRandomAccess.get).  An optional 'intensity' = (m00, m01) adjusts the view's
    values first (IntensityAdjuster).  Returns (image, weight) float32 [z][y][x]."""
    nx, ny, nz = bb_dims
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    s = np.stack([x + bb_min[0], y + bb_min[1], z + bb_min[2]], axis=-1).astype(np.float64)
    lut = blending_lut()
    sumI = np.zeros(s.shape[:-1])
    sumW = np.zeros(s.shape[:-1])
    sumD = np.zeros(s.shape[:-1])
    for v in views:
        img = np.asarray(v["img"], dtype=np.float32)
        if v.get("intensity") is not None:
            # IntensityAdjuster.apply (fusion/intensityadjust/IntensityAdjuster.java): v m00 + m01
            # in double, stored as float, before the interpolation
            m00, m01 = v["intensity"]
            img = (img.astype(np.float64) * m00 + m01).astype(np.float32)
        dims = (img.shape[2], img.shape[1], img.shape[0])
        inv = _invert_affine(v["model"])
        t = apply_affine(inv, s)
        tf = t.astype(np.float32)
        wf = blending_weight(tf, dims, *v["fusion"], lut=lut) if v.get("fusion") else np.ones(s.shape[:-1], np.float32)
        wd = blending_weight(tf, dims, *v["decon"], lut=lut) if v.get("decon") else np.ones(s.shape[:-1], np.float32)
        sumD += wd.astype(np.float64)
        inside = np.all((t > 0) & (t < np.array(dims, dtype=np.float64) - 1), axis=-1)
        val = np.zeros(s.shape[:-1], dtype=np.float32)
        acc = nlinear(lambda ix, iy, iz: img[iz, iy, ix], t[inside])
        val[inside] = np.maximum(np.float32(1), acc)
        use = wf != 0
        sumI += np.where(use, val.astype(np.float64) * wf.astype(np.float64), 0.0)
        sumW += np.where(use, wf.astype(np.float64), 0.0)
    image = np.where(sumW > 0, sumI / np.where(sumW > 0, sumW, 1.0), 0.0).astype(np.float32)
    return image, sumD.astype(np.float32)


# ---- PSF preparation (MV/process/psf, deconvolution/util/PSFPreparation.java) -------------
# Arrays [z][y][x] float32, sizes (x, y, z), models row-packed 3 x 4.

def _xyz(a):
    return (a.shape[2], a.shape[1], a.shape[0])


def _grid(size):
    z, y, x = np.meshgrid(np.arange(size[2]), np.arange(size[1]), np.arange(size[0]), indexing="ij")
    return x, y, z


def psf_extract(img, locations, size):
    """PSFExtraction.extractPSFLocal (MV/process/psf/PSFExtraction.java:234-269) on the
    periodic extension of img (the RandomAccessibleInterval constructors, :112-120): for each
    location l in order, every PSF voxel p adds the linear interpolation of the image at
    p - size / 2 + l (psf + value in double, stored as float)."""
    img = np.asarray(img, dtype=np.float32)
    D = _xyz(img)
    x, y, z = _grid(size)
    rel = np.stack([x - size[0] // 2, y - size[1] // 2, z - size[2] // 2], axis=-1).astype(np.float64)

    def get(ix, iy, iz):
        return img[np.mod(iz, D[2]), np.mod(iy, D[1]), np.mod(ix, D[0])]

    psf = np.zeros((size[2], size[1], size[0]), dtype=np.float32)
    for l in np.asarray(locations, dtype=np.float64).reshape(-1, 3):
        v = nlinear(get, rel + l)
        psf = (psf.astype(np.float64) + v.astype(np.float64)).astype(np.float32)
    return psf


def psf_normalize(psf):
    """PSFExtraction.normalize (:453-471): (v - min) / (max - min) in double, stored as float."""
    a = np.asarray(psf, dtype=np.float32).astype(np.float64)
    mn, mx = a.min(), a.max()
    with np.errstate(invalid="ignore", divide="ignore"):
        return ((a - mn) / (mx - mn)).astype(np.float32)


def psf_transformed_geometry(dims, model):
    """transformPSF's output size and offset (:367-409): the bounding box of the transformed
    corners of [0, dims - 1] (AffineTransform3D.estimateBounds), size (int) extent + 1 made
    odd, offset = model(dims / 2) - size / 2."""
    corners = np.array([[(c & 1) * (dims[0] - 1), ((c >> 1) & 1) * (dims[1] - 1), ((c >> 2) & 1) * (dims[2] - 1)]
                        for c in range(8)], dtype=np.float64)
    t = apply_affine(model, corners)
    lo, hi = t.min(axis=0), t.max(axis=0)
    center = apply_affine(model, np.array([d // 2 for d in dims], dtype=np.float64))
    size, off = [], []
    for d in range(3):
        n = int(hi[d] - lo[d]) + 1
        if n % 2 == 0:
            n += 1
        size.append(n)
        off.append(center[d] - (n // 2))
    return tuple(size), np.array(off)


def psf_transform_normalized(psf, model):
    """PSFExtraction.getTransformedNormalizedPSF (:182-188): normalize, then transform (:411-451):
    out(p) = linear interpolation of the zero-extended PSF at model^-1 (p + offset)."""
    p = psf_normalize(psf)
    dims = _xyz(p)
    size, off = psf_transformed_geometry(dims, model)
    inv = _invert_affine(model)
    x, y, z = _grid(size)
    s = np.stack([x + off[0], y + off[1], z + off[2]], axis=-1)
    t = apply_affine(inv, s)

    def get(ix, iy, iz):
        ok = (ix >= 0) & (iy >= 0) & (iz >= 0) & (ix < dims[0]) & (iy < dims[1]) & (iz < dims[2])
        v = p[np.clip(iz, 0, dims[2] - 1), np.clip(iy, 0, dims[1] - 1), np.clip(ix, 0, dims[0] - 1)]
        return np.where(ok, v, np.float32(0))

    return nlinear(get, t)


def psf_average(psfs, max_size=True):
    """PSFCombination.computeAverageImage (MV/process/psf/PSFCombination.java:74-138): the
    PSFs centred (centre = size / 2) on the largest or smallest size per axis, summed in float
    in list order, divided by their number (double)."""
    dl = [_xyz(p) for p in psfs]
    f = max if max_size else min
    a = tuple(f(d[k] for d in dl) for k in range(3))
    acc = np.zeros((a[2], a[1], a[0]), dtype=np.float32)
    for p, d in zip(psfs, dl):
        o = [a[k] // 2 - d[k] // 2 for k in range(3)]  # avg index of PSF voxel 0
        src = [slice(max(0, -o[k]), min(d[k], a[k] - o[k])) for k in range(3)]
        dst = [slice(max(0, o[k]), max(0, o[k]) + (src[k].stop - src[k].start)) for k in range(3)]
        acc[dst[2], dst[1], dst[0]] = (acc[dst[2], dst[1], dst[0]] +
                                       np.asarray(p, np.float32)[src[2], src[1], src[0]]).astype(np.float32)
    return (acc.astype(np.float64) / len(psfs)).astype(np.float32)


def psf_make_same_size(psf, size):
    """PSFCombination.makeSameSize (:182-210): the PSF centred in size, extended with its
    minimum."""
    p = np.asarray(psf, dtype=np.float32)
    d = _xyz(p)
    out = np.full((size[2], size[1], size[0]), np.float32(np.float64(p.min())), dtype=np.float32)
    x, y, z = _grid(size)
    px, py, pz = x - size[0] // 2 + d[0] // 2, y - size[1] // 2 + d[1] // 2, z - size[2] // 2 + d[2] // 2
    ok = (px >= 0) & (py >= 0) & (pz >= 0) & (px < d[0]) & (py < d[1]) & (pz < d[2])
    out[ok] = p[pz[ok], py[ok], px[ok]]
    return out


def psf_projection(psf, dim=-1, use_max=True):
    """PSFCombination.computeMaxProjection (:228-296): the max or min along axis dim (x = 0;
    dim < 0: the first smallest axis), the other axes kept in order.  Returns (projection
    [second kept][first kept], dim)."""
    p = np.asarray(psf, dtype=np.float32)
    d = _xyz(p)
    if dim < 0:
        dim = 0
        for k in range(1, 3):
            if d[k] < d[dim]:
                dim = k
    ax = 2 - dim  # numpy axis of (x, y, z) axis dim
    a = p.astype(np.float64)
    ext = np.full(np.delete(np.array(p.shape), ax), -np.finfo(np.float64).max if use_max else np.finfo(np.float64).max)
    for k in range(d[dim]):
        v = np.take(a, k, axis=ax)
        ext = np.where(v > ext, v, ext) if use_max else np.where(v < ext, v, ext)
    with np.errstate(over="ignore"):  # an all-NaN line keeps -+DBL_MAX, which rounds to -+inf
        return ext.astype(np.float32), dim


def psf_remove_min_projections(psf):
    """PSFExtraction.removeMinProjections / subtractProjection (:190-229): for axis 0, 1, 2 in
    turn the min projection along it is subtracted (float)."""
    p = np.array(psf, dtype=np.float32)
    for dim in range(3):
        proj, _ = psf_projection(p, dim, use_max=False)
        p = (p - np.expand_dims(proj, axis=2 - dim)).astype(np.float32)
    return p


def load_group_transform_psfs(groups, same_size_for_all=True):
    """PSFPreparation.loadGroupTransformPSFs (deconvolution/util/PSFPreparation.java:41-91):
    per group the average, on the smallest common size, of its views' normalised transformed
    PSFs; with same_size_for_all each is then centred in the largest size."""
    out = [psf_average([psf_transform_normalized(p, m) for p, m in grp], max_size=False) for grp in groups]
    if same_size_for_all:
        mx = tuple(max(_xyz(a)[k] for a in out) for k in range(3))
        out = [psf_make_same_size(a, mx) for a in out]
    return out
