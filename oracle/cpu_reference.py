"""Float32 CPU restatement of the reference block iteration with the reference's padded
real-to-complex FFT convolution: the timed CPU baseline.

TEST INFRASTRUCTURE ONLY: used by the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` (timed) and by tests/ (which pin it against the FP64-FFT C oracle in
mvr_oracle.c); never by the product library.

What it restates (paths relative to src/main/java/ of the reference,
MV = net/preibisch/mvrecon/process):

* ComputeBlockSeqThreadCPU.runIteration (MV/deconvolution/iteration/sequential/
  ComputeBlockSeqThreadCPU.java:79-169): conv1 of the mirror-single extended psi block
  (:171-189), the quotient, conv2 of the value-1 extended quotient (:191-209), the update;
* util/FFTConvolution.java:508-603 (setupFFTs, computeImgFFT, computeKernelFFT,
  computeConvolution): the input padded to a "fast" size >= block + kernel - 1, the block
  centred in it (paddingIntervalCentered), the kernel zero-extended with its centre
  voxel at the origin (periodic wrap), a float real-to-complex transform, the complex
  product, the complex-to-real transform and the centred crop (complexToRealUnpad);
* DeconvolutionMethods.computeQuotient / computeNextValue / tikhonov
  (MV/deconvolution/iteration/sequential/DeconvolutionMethods.java:46-98, 320-358, 421)
  in float32 with the Tikhonov factor in double, as Java evaluates them;
* Block.copyBlock / pasteBlock (MV/cuda/Block.java:158-239): mirror-single extraction of
  psi from the whole volume, zero extension of image and weight, paste of the effective
  region (MultiViewDeconvolutionSeq.java:115-143).

The FFT arithmetic of the reference is imglib2-algorithm-fft's FFT / FFTMethods over the
Mines JTK FFT (managed by org.scijava:pom-scijava 43.0.0, not vendored).  Its published
algorithm is a prime-factor FFT whose lengths are products of mutually prime factors
from {2, 3, 4, 5, 7, 8, 9, 11, 13, 16}, i.e. 2^a 3^b 5^c 7^d 11^e 13^f with a <= 4,
b <= 2 and c, d, e, f <= 1; the real transform of the first axis runs a complex one of
half its (even) length.  FFTMethods.dimensionsRealToComplexFast picks such lengths;
here every axis takes the smallest valid length >= block + kernel - 1 (JTK's own
cost-table choice can be larger).  The transforms themselves are pocketfft's single
precision real-to-complex transforms (scipy.fft, all host threads): a faster CPU FFT
than the reference's, so the baseline errs on the fast side.  The padded size does not
change the updated block beyond float rounding (the linear convolution of the extended
block is the same for every padding >= block + kernel - 1).
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

try:
    import scipy.fft as _sfft
except Exception:  # pragma: no cover - scipy is on both machines
    _sfft = None


def cores() -> int:
    return os.cpu_count() or 1


def _rfftn(a, workers):
    if _sfft is not None:
        return _sfft.rfftn(a, workers=workers)
    return np.fft.rfftn(a)


def _irfftn(a, s, workers):
    if _sfft is not None:
        return _sfft.irfftn(a, s=s, workers=workers)
    return np.fft.irfftn(a, s=s)


def jtk_valid(n: int) -> bool:
    """n = 2^a 3^b 5^c 7^d 11^e 13^f with a <= 4, b <= 2, c..f <= 1 (the lengths of a
    prime-factor FFT over the mutually prime factors 2/4/8/16, 3/9, 5, 7, 11, 13)."""
    if n < 1:
        return False
    for p, emax in ((2, 4), (3, 2), (5, 1), (7, 1), (11, 1), (13, 1)):
        e = 0
        while n % p == 0:
            n //= p
            e += 1
        if e > emax:
            return False
    return n == 1


def fft_size_complex(n: int) -> int:
    while not jtk_valid(n):
        n += 1
    return n


def fft_size_real(n: int) -> int:
    """Even length whose half is a valid complex length."""
    h = (n + 1) // 2
    while not jtk_valid(h):
        h += 1
    return 2 * h


def padded_domain(block_xyz, kernel_xyz):
    """(Px, Py, Pz): the real axis x and the complex axes y, z at the smallest valid
    lengths >= block + kernel - 1."""
    n = [block_xyz[d] + kernel_xyz[d] - 1 for d in range(3)]
    return fft_size_real(n[0]), fft_size_complex(n[1]), fft_size_complex(n[2])


def mirror_single(i: np.ndarray, n: int) -> np.ndarray:
    """Mirror extension with a single boundary (period 2n - 2, the border voxel once)."""
    if n <= 1:
        return np.zeros_like(i)
    p = 2 * n - 2
    i = np.mod(i, p)
    return np.where(i >= n, p - i, i)


class PaddedConvolver:
    """util/FFTConvolution for one block size and one kernel: the kernel spectrum is
    computed once and kept (DeconViewPSF.getKernel1FFT / getKernel2FFT cache it per
    block size, DeconViewPSF.java:79-111)."""

    def __init__(self, block_xyz, kernel, workers=None):
        self.workers = workers or cores()
        self.b = tuple(int(v) for v in block_xyz)
        kd = (kernel.shape[2], kernel.shape[1], kernel.shape[0])
        self.P = padded_domain(self.b, kd)
        P = self.P
        # paddingIntervalCentered: the block starts at (P - b) / 2 of the padded domain
        self.lo = tuple((P[d] - self.b[d]) // 2 for d in range(3))
        # the kernel zero-extended, its centre voxel k / 2 at the origin (periodic wrap)
        kp = np.zeros((P[2], P[1], P[0]), dtype=np.float32)
        iz = np.mod(np.arange(kd[2]) - kd[2] // 2, P[2])
        iy = np.mod(np.arange(kd[1]) - kd[1] // 2, P[1])
        ix = np.mod(np.arange(kd[0]) - kd[0] // 2, P[0])
        kp[np.ix_(iz, iy, ix)] = np.asarray(kernel, dtype=np.float32)
        self.K = _rfftn(kp, self.workers)
        # padded index -> block index under mirror-single extension
        self.mirror = [mirror_single(np.arange(P[d]) - self.lo[d], self.b[d]) for d in range(3)]

    def __call__(self, block, ext_value=None):
        """Linear convolution of the block extended by mirror-single (ext_value None) or
        by a constant, output over the block (float32)."""
        P, lo, b = self.P, self.lo, self.b
        if ext_value is None:
            a = block[np.ix_(self.mirror[2], self.mirror[1], self.mirror[0])]
        else:
            a = np.full((P[2], P[1], P[0]), ext_value, dtype=np.float32)
            a[lo[2]:lo[2] + b[2], lo[1]:lo[1] + b[1], lo[0]:lo[0] + b[0]] = block
        A = _rfftn(a, self.workers)
        A *= self.K
        y = _irfftn(A, (P[2], P[1], P[0]), self.workers)
        return np.ascontiguousarray(y[lo[2]:lo[2] + b[2], lo[1]:lo[1] + b[1], lo[0]:lo[0] + b[0]], dtype=np.float32)


def _chunks(n, parts):
    step = max(1, (n + parts - 1) // parts)
    return [(s, min(n, s + step)) for s in range(0, n, step)]


def _update_slab(psi, conv2, w, lam, min_value, max_intensity):
    """computeNextValue over a slab (float32, Tikhonov in double); returns the signed
    change sum (double) and max."""
    minI = np.float32(min_value)
    maxI = np.float32(max_intensity)
    last = psi.copy()
    value = last * conv2
    pos = value > 0
    if lam > 0:
        v = (value / maxI).astype(np.float64)
        tik = ((np.sqrt(1.0 + 2.0 * lam * v) - 1.0) / lam).astype(np.float32)
        adjusted = np.where(pos, tik * maxI, minI)
    else:
        adjusted = np.where(pos, value, minI)
    nxt = np.where(np.isnan(adjusted), minI, np.maximum(minI, adjusted)).astype(np.float32)
    psi[...] = last + (nxt - last) * w
    ch = psi - last
    return float(ch.sum(dtype=np.float64)), float(ch.max()) if ch.size else -1.0


def block_seq(psi, img, w, conv1, conv2, lam, min_value, max_intensity, pool=None, parts=1):
    """ComputeBlockSeqThreadCPU.runIteration on one block, in place on psi (float32);
    conv1 / conv2 are PaddedConvolver objects of kernel1 / kernel2; the update runs in
    `parts` z-slabs on `pool`.  Returns (sum, max) of the signed change
    (IterationStatistics)."""
    blurred = conv1(psi)
    # computeQuotient: img > 0 ? img / blurred : 1 (no epsilon)
    with np.errstate(divide="ignore", invalid="ignore"):
        q = np.where(img > 0, img / blurred, np.float32(1)).astype(np.float32)
    c2 = conv2(q, 1.0)
    if pool is None or parts <= 1:
        res = [_update_slab(psi, c2, w, lam, min_value, max_intensity)]
    else:
        res = list(pool.map(lambda r: _update_slab(psi[r[0]:r[1]], c2[r[0]:r[1]], w[r[0]:r[1]], lam, min_value,
                                                   max_intensity), _chunks(psi.shape[0], parts)))
    return sum(r[0] for r in res), max([-1.0] + [r[1] for r in res])


def extract(vol, off_xyz, b_xyz, mode):
    """Block.copyBlock: the block at off of a [z][y][x] volume, mirror-single ('mirror')
    or zero ('zero') outside it."""
    D = (vol.shape[2], vol.shape[1], vol.shape[0])
    idx = [np.arange(off_xyz[d], off_xyz[d] + b_xyz[d]) for d in range(3)]
    if mode == "mirror":
        m = [mirror_single(idx[d], D[d]) for d in range(3)]
        return np.ascontiguousarray(vol[np.ix_(m[2], m[1], m[0])], dtype=np.float32)
    out = np.zeros((b_xyz[2], b_xyz[1], b_xyz[0]), dtype=np.float32)
    ok = [(idx[d] >= 0) & (idx[d] < D[d]) for d in range(3)]
    if all(o.any() for o in ok):
        src = np.ix_(idx[2][ok[2]], idx[1][ok[1]], idx[0][ok[0]])
        dst = np.ix_(np.nonzero(ok[2])[0], np.nonzero(ok[1])[0], np.nonzero(ok[0])[0])
        out[dst] = vol[src]
    return out


def paste(vol, blk, eff_offset, eff_size, eff_local):
    """Block.pasteBlock: the effective region back into the volume."""
    eo, es, el = eff_offset, eff_size, eff_local
    vol[eo[2]:eo[2] + es[2], eo[1]:eo[1] + es[1], eo[0]:eo[0] + es[0]] = \
        blk[el[2]:el[2] + es[2], el[1]:el[1] + es[1], el[0]:el[0] + es[0]]


class BlockSampler:
    """A bounded sample of the sequential deconvolution of a whole volume on the host
    cores: every step takes one block of each view's grid (block j of step j, views in
    order, MultiViewDeconvolutionSeq.runNextIteration's view order) and pastes its
    effective region back into psi before the next view, so the sampled blocks iterate
    on real psi.  voxel_iterations counts what the step advanced: each view-block moves
    its effective region by one view's share (1 / V) of an iteration."""

    def __init__(self, psi, images, weights, k1s, k2s, grids, block_xyz, lam, max_intensities, min_value=1e-4,
                 workers=None, image_block=None, weight_block=None):
        """images / weights: per view [z][y][x] arrays (normalised weights), or None when
        image_block(v, offset, b) / weight_block(v, offset, b) give the zero-extended
        blocks instead."""
        self.psi = psi
        self.k1s, self.k2s = k1s, k2s
        self.grids = grids  # per view: list of dicts (offset, eff_offset, eff_size, eff_local)
        self.views = len(grids)
        # one block size (x, y, z) for every view, or a list with one per view
        per_view = isinstance(block_xyz[0], (tuple, list))
        self.bs = [tuple(b) for b in block_xyz] if per_view else [tuple(block_xyz)] * self.views
        self.b = self.bs[0]
        self.lam, self.mx, self.min_value = lam, list(max_intensities), min_value
        self.image_block = image_block or (lambda v, off, b: extract(images[v], off, b, "zero"))
        self.weight_block = weight_block or (lambda v, off, b: extract(weights[v], off, b, "zero"))
        self.workers = workers or cores()
        self.pool = cf.ThreadPoolExecutor(max_workers=self.workers)
        self.conv = {}
        self.step_index = 0

    def close(self):
        self.pool.shutdown()

    def _convolvers(self, v):
        if v not in self.conv:
            self.conv[v] = (PaddedConvolver(self.bs[v], self.k1s[v], self.workers),
                            PaddedConvolver(self.bs[v], self.k2s[v], self.workers))
        return self.conv[v]

    def prepare(self):
        """Kernel spectra of every view (set-up, outside any timed region)."""
        for v in range(self.views):
            self._convolvers(v)

    def step(self):
        V = self.views
        advanced = 0.0
        for v in range(V):
            grid = self.grids[v]
            bl = grid[self.step_index % len(grid)]
            c1, c2 = self._convolvers(v)
            b = self.bs[v]
            p = extract(self.psi, bl["offset"], b, "mirror")
            img = self.image_block(v, bl["offset"], b)
            w = self.weight_block(v, bl["offset"], b)
            block_seq(p, img, w, c1, c2, self.lam, self.min_value, self.mx[v], self.pool, self.workers)
            paste(self.psi, p, bl["eff_offset"], bl["eff_size"], bl["eff_local"])
            es = bl["eff_size"]
            advanced += float(es[0]) * es[1] * es[2] / V
        self.step_index += 1
        return advanced
