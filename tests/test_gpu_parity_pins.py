"""GPU parity against the CPU oracle where the benchmark runs and where the fast paths
take their shortcuts (all through the C ABI):

* one full-size view-block of the 4-view 256^3 workload: a 192^3 block with the
  31x31x61 Optimization-I kernels, circular boundary, i.e. the 192 x 192 plane kernels
  and the 192-long Z pass the benchmark runs, two view-steps in a row; effective
  region within relative L2 1e-5 of the reference-faithful oracle after each;
* the reference's 2-view 128x128x64 case end to end (PSF 15x15x31 at 0 / 90 degrees,
  efficient-Bayesian kernels, all-one weights, one block, 10 iterations): within 1e-4
  of the oracle after every iteration and of the FP64 oracle after 10, on the plane
  kernels (192x192x128 block, circular) and on the reference boundary (156x156x124);
* the update guards on a plane-kernel shape (128x128x64): psi = 0 (value 0 -> minI),
  psi > 0 with a negative conv2 (value < 0 -> minI), NaN and negative image values
  (quotient 1), a negative conv1 with image data (no epsilon), and maxIntensity = +Inf
  (the Tikhonov value is NaN -> minI); guarded voxels must come out exactly
  psi + (minI - psi) w in float;
* the multiplicative update with conv2 values whose float product leaves the float
  range (the reference multiplies in double);
* smooth weights and OSEM != 1 against the oracle's NormalizingRandomAccess;
* a volume whose weight is zero over a whole block, which filterBlocksForContent drops,
  so the batch-order path runs; against the oracle's driver.
"""
import numpy as np
import pytest

import mvrgb300 as M
import oracle as O
import synthetic

pytestmark = pytest.mark.gpu
MIN_I = np.float32(1e-4)


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def guarded(psi, w):
    """psi + (minI - psi) * w in float32 (computeNextValue with adjustedValue = minI)."""
    psi = np.asarray(psi, np.float32)
    w = np.asarray(w, np.float32)
    return (psi + (MIN_I - psi) * w).astype(np.float32)


# ---- (a) a full-size view-block of the headline workload --------------------------------

def test_headline_view_block_on_plane_kernels_against_oracle():
    psfs = [synthetic.make_psf((31, 31, 61), 1.5, 4.5, a, side_lobes=True) for a in (0.0, 45.0, 90.0, 135.0)]
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    b = (192, 192, 192)
    rng = np.random.default_rng(192)
    shape = b[::-1]
    psi = rng.uniform(20, 200, shape).astype(np.float32)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < 0.03] = 0
    ws = [rng.uniform(0, 1, shape).astype(np.float32) for _ in range(2)]
    e = [30, 30, 60]  # k - 1 on each side: the effective region 132 x 132 x 72
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    ref = psi.copy()
    out = psi.copy()
    with M.BlockWorker(b, 1e-4, 0.006, 2, M.BOUNDARY_CIRCULAR) as wk:  # kernels of two views
        for v in range(2):
            wk.set_kernels(v, k1s[v], k2s[v])
        for v in range(2):
            ref, _ = O.block_seq(ref, img, ws[v], k1s[v], k2s[v], 0.006, 1e-4, 300.0)
            wk.run_iteration(v, out, img, ws[v], 300.0)
            # the circular block's margin differs; the effective region is what is pasted
            assert rel(out[sl], ref[sl]) <= 1e-5, v
            out[:] = ref  # the next view-step starts from the same psi on both sides


# ---- (b) the 2-view 128x128x64 case end to end ------------------------------------------

@pytest.fixture(scope="module")
def small():
    ds = synthetic.config_small()
    k1s, k2s = O.psf_init(ds.psfs, O.PSF_EFFICIENT_BAYESIAN, 0)
    psi0, mx, _ = O.psi_init_avg(ds.images)
    return ds, k1s, k2s, psi0, mx


@pytest.mark.parametrize("block,boundary", [((192, 192, 128), M.BOUNDARY_CIRCULAR),
                                            ((156, 156, 124), M.BOUNDARY_REFERENCE)])
def test_two_view_case_ten_iterations_against_oracle(small, block, boundary):
    ds, k1s, k2s, psi0, mx = small
    ones = [np.ones_like(ds.images[0]) for _ in range(2)]
    ref = psi0
    errs = []
    with M.Deconvolution((128, 128, 64), 2, block, psf_type=M.PSF_EFFICIENT_BAYESIAN, psf_norm_threads=0, lam=0.0,
                         boundary=boundary, weight_norm=M.WEIGHTS_AS_GIVEN) as d:
        for v in range(2):
            d.set_view(v, ds.images[v], ones[v], ds.psfs[v])
        d.prepare()
        assert np.array_equal(d.max_intensities(), mx)
        assert np.array_equal(d.get_psi(), psi0)
        for it in range(10):
            d.run_iterations(1)
            # the oracle's one block: image + 2 (k - 1) per axis
            ref, _ = O.decon_run(ref, ds.images, ones, k1s, k2s, (156, 156, 124), 1, lam=0.0, max_intensities=mx)
            errs.append(rel(d.get_psi(), ref))
            assert errs[-1] <= 1e-4, (it, errs)
        psi = d.get_psi()
    ref64, _ = O.decon_run(psi0, ds.images, ones, k1s, k2s, (156, 156, 124), 10, lam=0.0, max_intensities=mx,
                           fp64=True)
    assert rel(psi, ref64) <= 1e-4


# ---- (c) update guards on a plane-kernel shape ------------------------------------------

def guard_case():
    b, kd = (128, 128, 64), (9, 9, 15)
    rng = np.random.default_rng(11)
    shape = b[::-1]
    k1 = synthetic.make_psf(kd, 1.2, 2.5, 30.0)
    k2 = O.invert_kernel(k1)
    psi = rng.uniform(20, 200, shape).astype(np.float32)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    w = rng.uniform(0.1, 1, shape).astype(np.float32)
    r = [k // 2 + 1 for k in kd]  # kernel radius + 1 (x, y, z)
    # a slab of psi = 0 without image data: quotient 1, value = 0 * conv2 = 0 -> minI
    zs = slice(24, 40)
    psi[zs, 10:50, 10:50] = 0.0
    img[zs.start - r[2]:zs.stop + r[2], 10 - r[1]:50 + r[1], 10 - r[0]:50 + r[0]] = 0.0
    # a box of psi = -5 with image data inside (conv1 < 0: the quotient has no epsilon),
    # no image data in a shell around its face (conv1 crosses zero there)
    bz, by, bx = slice(16, 48), slice(70, 118), slice(70, 118)
    psi[bz, by, bx] = -5.0
    shell = np.zeros(shape, bool)
    shell[bz.start - r[2]:bz.stop + r[2], by.start - r[1]:by.stop + r[1], bx.start - r[0]:bx.stop + r[0]] = True
    shell[bz.start + r[2]:bz.stop - r[2], by.start + r[1]:by.stop - r[1], bx.start + r[0]:bx.stop - r[0]] = False
    img[shell] = 0.0
    # one positive psi voxel inside it: conv2 < 0 there, so value < 0 -> minI
    pz, py, px = 32, 94, 94
    psi[pz, py, px] = 3.0
    # NaN and negative image values: img > 0 fails, quotient 1
    nan_at = (rng.integers(0, 64, 40), rng.integers(0, 60, 40), rng.integers(0, 60, 40))
    img[nan_at] = np.nan
    img[rng.integers(0, 64, 40), rng.integers(0, 60, 40), rng.integers(0, 60, 40)] = -7.0
    return b, kd, psi, img, w, k1, k2, zs, (pz, py, px)


def test_update_guards_on_plane_kernels():
    b, kd, psi, img, w, k1, k2, zs, pv = guard_case()
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    with M.BlockWorker(b, 1e-4, 0.006, 1, M.BOUNDARY_CIRCULAR) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        wk.run_iteration(0, out, img, w, 300.0)
    assert np.isfinite(out).all() and np.isfinite(ref).all()
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    assert rel(out[sl], ref[sl]) <= 1e-5
    # guarded voxels are exact
    zero = psi == 0.0
    assert zero.sum() > 10000
    assert np.array_equal(out[zero], guarded(psi[zero], w[zero]))
    assert np.array_equal(ref[zero], guarded(psi[zero], w[zero]))
    assert out[pv] == guarded(psi[pv], w[pv]) == ref[pv]
    # the reference boundary (FFT domain >= block + kernel - 1) on the same block agrees
    # with the oracle on the whole block
    with M.BlockWorker((114, 114, 50), 1e-4, 0.006, 1, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, k1, k2)
        sub = (slice(7, 57), slice(7, 121), slice(7, 121))
        out2 = np.ascontiguousarray(psi[sub])
        wk.run_iteration(0, out2, np.ascontiguousarray(img[sub]), np.ascontiguousarray(w[sub]), 300.0)
    ref2, _ = O.block_seq(psi[sub], img[sub], w[sub], k1, k2, 0.006, 1e-4, 300.0)
    assert np.isfinite(out2).all()
    assert rel(out2, ref2) <= 1e-5
    z2 = psi[sub] == 0.0
    assert np.array_equal(out2[z2], ref2[z2])


def test_nan_tikhonov_value_gives_min_intensity():
    # maxIntensity = +Inf: value / max = 0, tikhonov 0, 0 * Inf = NaN -> minI for value > 0,
    # minI for value <= 0 too: every voxel becomes psi + (minI - psi) w
    b, kd, psi, img, w, k1, k2, _, _ = guard_case()
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, float("inf"))
    with M.BlockWorker(b, 1e-4, 0.006, 1, M.BOUNDARY_CIRCULAR) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        wk.run_iteration(0, out, img, w, float("inf"))
    assert np.array_equal(out, guarded(psi, w))
    assert np.array_equal(ref, guarded(psi, w))


# ---- the multiplicative update beyond the float range of the product --------------------

@pytest.mark.parametrize("b", [(128, 128, 64), (40, 36, 44)])  # plane kernels, row kernels
def test_mul_product_beyond_float_range(b):
    # psi tiny (1e-8) under bright images: conv1 ~ 1e-8, quotient ~ 1e10 and conv2 ~ 1e10
    # in 4 views; their product (~1e40) overflows float, the reference's double does not.
    # The whole block is tiny: a float FFT (the reference's too) cannot resolve values of
    # order 1 next to values of order 1e10 in one block.
    rng = np.random.default_rng(3)
    shape = b[::-1]
    kd = (5, 5, 7)
    k1s = [synthetic.make_psf(kd, 1.0, 1.5, a) for a in (0.0, 45.0, 90.0, 135.0)]
    k2s = [O.invert_kernel(k) for k in k1s]
    psi = rng.uniform(0.5e-8, 2e-8, shape).astype(np.float32)
    imgs = [rng.uniform(50, 300, shape).astype(np.float32) for _ in range(4)]
    ws = [rng.uniform(0.1, 1, shape).astype(np.float32) for _ in range(4)]
    mx = [300.0] * 4
    ref, _ = O.block_mul(psi, imgs, ws, k1s, k2s, 0.006, 1e-4, mx)
    with M.BlockWorker(b, 1e-4, 0.006, 4, M.BOUNDARY_CIRCULAR) as wk:
        for v in range(4):
            wk.set_kernels(v, k1s[v], k2s[v])
        out = psi.copy()
        wk.run_iteration_mul(out, imgs, ws, mx)
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    assert np.isfinite(out).all()
    assert rel(out[sl], ref[sl]) <= 1e-5
    # every voxel rises from 1e-8 to about the image level through the product; a float
    # product would overflow and give minI instead
    assert (ref[sl] > 1.0).all() and (out[sl] > 1.0).all()


# ---- weight normalisation variants ------------------------------------------------------

@pytest.mark.parametrize("norm,osem", [(M.WEIGHTS_SMOOTH, 1.0), (M.WEIGHTS_HARD, 2.5), (M.WEIGHTS_SMOOTH, 3.0)])
def test_weight_normalisation_variants_against_oracle(norm, osem):
    rng = np.random.default_rng(5)
    dims = (40, 36, 30)
    shape = dims[::-1]
    raws = [rng.uniform(0, 1.3, shape).astype(np.float32) for _ in range(3)]
    for r in raws:
        r[rng.random(shape) < 0.1] = 0.0
    imgs = [rng.uniform(5, 100, shape).astype(np.float32) for _ in range(3)]
    psf = synthetic.make_psf((5, 5, 7), 1.0, 1.5, 0.0)
    smooth = norm == M.WEIGHTS_SMOOTH
    ref = O.normalize_weights(raws, osem=osem, smooth=smooth, max_diff_range=0.1, scaling_range=0.05)
    with M.Deconvolution(dims, 3, (28, 28, 28), weight_norm=norm, osem_speedup=osem, max_diff_range=0.1,
                         scaling_range=0.05) as d:
        for v in range(3):
            d.set_view(v, imgs[v], raws[v], psf)
        d.prepare()
        for v in range(3):
            got = d.weights(v)
            assert np.abs(got - ref[v]).max() <= 1e-6, v


# ---- a weight-empty block dropped by filterBlocksForContent ------------------------------

def test_weight_empty_block_is_dropped_and_batch_order_runs():
    rng = np.random.default_rng(9)
    dims = (40, 36, 30)
    shape = dims[::-1]
    psfs = [synthetic.make_psf((5, 5, 7), 1.0, 1.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 100, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    block = (20, 20, 20)
    # view 0's weight is zero over the first block's whole box (offset -(2k-1-1)/2 per axis)
    kk = [2 * k - 1 for k in (5, 5, 7)]
    blocks = O.divide_into_blocks(dims, kk, block)
    off = blocks[0]["offset"]
    box = tuple(slice(max(0, off[d]), off[d] + block[d]) for d in (2, 1, 0))
    ws[0][box] = 0.0
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, block, 2, lam=0.006, max_intensities=mx, filter_blocks=True)
    with M.Deconvolution(dims, 2, block, psf_type=M.PSF_OPTIMIZATION_I, psf_norm_threads=0, lam=0.006,
                         weight_norm=M.WEIGHTS_AS_GIVEN, filter_blocks=True) as d:
        for v in range(2):
            d.set_view(v, imgs[v], ws[v], psfs[v])
        d.prepare()
        d.run_iterations(2)
        psi = d.get_psi()
    assert rel(psi, ref) <= 1e-4
    # the same volume without the filter (every block kept: the Jacobi form of the step)
    unfiltered, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, block, 2, lam=0.006, max_intensities=mx,
                                filter_blocks=False)
    with M.Deconvolution(dims, 2, block, psf_type=M.PSF_OPTIMIZATION_I, psf_norm_threads=0, lam=0.006,
                         weight_norm=M.WEIGHTS_AS_GIVEN, filter_blocks=False) as d:
        for v in range(2):
            d.set_view(v, imgs[v], ws[v], psfs[v])
        d.prepare()
        d.run_iterations(2)
        assert rel(d.get_psi(), unfiltered) <= 1e-4


# ---- per-view compute blocks (DeconView takes its block size per view) -------------------

def test_per_view_block_sizes_against_one_block_oracle():
    # effective blocks of 16 voxels plus each view's overlap; with every effective region at
    # least k - 1 along the slab axis the blocked result equals the one-block result
    rng = np.random.default_rng(12)
    dims = (48, 40, 36)
    shape = dims[::-1]
    ks = [(5, 5, 7), (7, 7, 9), (9, 9, 11)]
    psfs = [synthetic.make_psf(k, 1.0, 1.5, a) for k, a in zip(ks, (0.0, 60.0, 120.0))]
    imgs = [rng.uniform(5, 100, shape).astype(np.float32) for _ in range(3)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(3)]
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    one = (64, 56, 56)  # one block for every view
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, one, 2, lam=0.006, max_intensities=mx)
    with M.Deconvolution(dims, 3, one, psf_type=M.PSF_OPTIMIZATION_I, psf_norm_threads=0, lam=0.006,
                         weight_norm=M.WEIGHTS_AS_GIVEN, boundary=M.BOUNDARY_REFERENCE) as d:
        for v in range(3):
            d.set_view(v, imgs[v], ws[v], psfs[v])
            d.set_view_block_size(v, tuple(16 + 2 * (ks[v][i] - 1) for i in range(3)))
        d.prepare()
        d.run_iterations(2)
        psi = d.get_psi()
    assert rel(psi, ref) <= 1e-4
