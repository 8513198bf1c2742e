"""The float32 CPU baseline (oracle/cpu_reference.py: padded real-to-complex FFT
convolution as util/FFTConvolution does it) pinned against the FP64-FFT C oracle.

Tolerances: the convolutions within 1e-6 relative L2 of the oracle's; a block
iteration within 1e-5 (the GPU's per-iteration bar); one sampled step of the whole
volume driver within 1e-5 of the oracle's driver on a one-block volume.
"""
import numpy as np
import pytest

import cpu_reference as R
import oracle as O
import synthetic


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fft_length_rule():
    valid = [n for n in range(1, 60) if R.jtk_valid(n)]
    assert valid == [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 18, 20, 21, 22, 24, 26, 28, 30, 33, 35,
                     36, 39, 40, 42, 44, 45, 48, 52, 55, 56]
    assert not R.jtk_valid(32) and not R.jtk_valid(27) and not R.jtk_valid(25) and R.jtk_valid(720720)
    # the 4-view 256^3 workload's 192^3 blocks with 31x31x61 kernels: 222 x 222 x 252
    assert R.padded_domain((192, 192, 192), (31, 31, 61)) == (224, 231, 252)
    for n in range(2, 400):
        p = R.fft_size_real(n)
        assert p >= n and p % 2 == 0 and R.jtk_valid(p // 2)
        assert R.fft_size_complex(n) >= n and R.jtk_valid(R.fft_size_complex(n))


@pytest.mark.parametrize("b,kd", [((40, 36, 44), (9, 7, 11)), ((33, 20, 17), (5, 9, 3))])
def test_padded_convolutions_against_oracle(b, kd):
    rng = np.random.default_rng(sum(b))
    blk = rng.uniform(0, 10, b[::-1]).astype(np.float32)
    k = rng.uniform(0, 1, kd[::-1]).astype(np.float32)
    c = R.PaddedConvolver(b, k, workers=2)
    assert rel(c(blk), O.convolve(blk, k, O.EXT_MIRROR_SINGLE)) <= 1e-6
    assert rel(c(blk, 1.0), O.convolve(blk, k, O.EXT_VALUE, 1.0)) <= 1e-6


@pytest.mark.parametrize("lam", [0.006, 0.0])
def test_block_iteration_against_oracle(lam):
    rng = np.random.default_rng(1)
    b = (40, 36, 44)
    shape = b[::-1]
    k1 = synthetic.make_psf((9, 7, 11), 1.0, 2.0, 30.0)
    k2 = O.invert_kernel(k1)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < 0.05] = 0
    w = rng.uniform(0, 1, shape).astype(np.float32)
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    ref, st = O.block_seq(psi, img, w, k1, k2, lam, 1e-4, 300.0)
    p = psi.copy()
    s, m = R.block_seq(p, img, w, R.PaddedConvolver(b, k1, 2), R.PaddedConvolver(b, k2, 2), lam, 1e-4, 300.0)
    assert rel(p, ref) <= 1e-5
    assert abs(m - st[1]) <= 1e-4 * max(1.0, abs(st[1]))


def test_sampler_step_is_one_driver_iteration_on_a_one_block_volume():
    rng = np.random.default_rng(4)
    dims = (24, 20, 18)
    shape = dims[::-1]
    psfs = [synthetic.make_psf((5, 5, 7), 1.0, 1.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 100, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    psi0 = (psi0 * rng.uniform(0.5, 1.5, shape)).astype(np.float32)  # not a constant
    block = (40, 36, 34)  # one block: image + 2 (k - 1) per axis or more
    grids = [O.divide_into_blocks(dims, [2 * k - 1 for k in (5, 5, 7)], block) for _ in range(2)]
    assert len(grids[0]) == 1
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, block, 1, lam=0.006, max_intensities=mx)
    s = R.BlockSampler(psi0.copy(), imgs, ws, k1s, k2s, grids, block, 0.006, mx, workers=2)
    try:
        adv = s.step()
    finally:
        s.close()
    assert adv == dims[0] * dims[1] * dims[2]  # every voxel advanced by one iteration
    assert rel(s.psi, ref) <= 1e-5
