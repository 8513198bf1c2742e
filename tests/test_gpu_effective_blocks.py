"""Compute blocks with more overlap than the kernel needs (an effective block size set on
the whole-volume driver), and the 288-long tile columns (18 x 16) that such blocks use
along z.  Through the C ABI.

Tolerances as elsewhere: relative L2 1e-5 per block iteration against the oracle on the
effective region, 1e-6 between two GPU paths on the same inputs (float rounding only), 1e-4
after two whole-volume iterations against the oracle's driver.
"""
import contextlib
import os

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O
import synthetic

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@contextlib.contextmanager
def env(**kv):
    old = {k: os.environ.get(k) for k in kv}
    os.environ.update({k: str(v) for k, v in kv.items()})
    try:
        yield
    finally:
        for k, v in old.items():
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def test_288_tile_columns_block_against_oracle():
    # a 128 x 128 x 288 circular block: z in two-phase tile columns of 18 x 16, on the plane
    # kernels and on the row / column kernels
    b, kd = (128, 128, 288), (9, 9, 15)
    rng = np.random.default_rng(288)
    shape = b[::-1]
    k1 = synthetic.make_psf(kd, 1.2, 2.5, 35.0)
    k2 = O.invert_kernel(k1)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < 0.05] = 0
    w = rng.uniform(0, 1, shape).astype(np.float32)
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    out = {}
    for plane in (1, 0):
        with env(MVR_PLANE_KERNELS=plane), M.BlockWorker(b, 1e-4, 0.006, 1, M.BOUNDARY_CIRCULAR) as wk:
            wk.set_kernels(0, k1, k2)
            p = psi.copy()
            st = wk.run_iteration(0, p, img, w, 300.0)
            out[plane] = (p, st)
    assert np.isfinite(out[1][0]).all()
    assert rel(out[1][0], out[0][0]) <= 1e-6
    assert out[1][1].max_change == pytest.approx(out[0][1].max_change, rel=1e-5, abs=1e-5)
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    for plane in (1, 0):
        assert rel(out[plane][0][sl], ref[sl]) <= 1e-5


def test_forced_schedules_on_288_columns():
    # 192 x 192 x 288 blocks: single-CTA and pair plane kernels, z through the tile-column
    # kernels and the persistent z pipeline, all on 288-long columns
    rng = np.random.default_rng(5)
    dims = (200, 190, 300)
    shape = dims[::-1]
    psfs = [synthetic.make_psf((9, 9, 15), 1.2, 2.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 200, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    codes = [M.SCHED_ROWS, M.SCHED_ROWS | M.SCHED_ZPIPE, M.SCHED_PLANE, M.SCHED_PLANE | M.SCHED_ZPIPE,
             M.SCHED_PLANE_PERSIST, M.SCHED_PAIR, M.SCHED_PAIR | M.SCHED_ZPIPE]
    out = {}
    for code in codes:
        with M.Deconvolution(dims, 2, (192, 192, 288), psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                             boundary=M.BOUNDARY_CIRCULAR, weight_norm=M.WEIGHTS_AS_GIVEN) as d:
            for v in range(2):
                d.set_view(v, imgs[v], ws[v], psfs[v])
            d.set_schedule(code)
            d.prepare()
            assert d.schedule(0) == code
            d.run_iterations(2)
            out[code] = d.get_psi()
    for code in codes:
        assert np.isfinite(out[code]).all()
        assert rel(out[code], out[M.SCHED_ROWS]) <= 1e-6, M.schedule_name(code)


@pytest.mark.parametrize("mul", [False, True])
def test_effective_block_grid_matches_the_reference_grid(mul):
    # effective blocks 48 x 40 x 36 with 9 x 9 x 15 PSFs: the reference's blocks are
    # 64 x 56 x 64 (effective + 2 (k - 1)); here 128 x 128 x 96 compute blocks (plane kernels)
    # on the same grid of effective blocks, and the same effective size with the reference's
    # own block size
    rng = np.random.default_rng(48)
    dims = (150, 130, 100)
    shape = dims[::-1]
    psfs = [synthetic.make_psf((9, 9, 15), 1.2, 2.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 200, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    for w in ws:
        # no weight from x = 120 on: the reference drops the blocks at x 144 ... 149, whose
        # own blocks (x 136 ... 199) hold no weight, although a 128-wide compute block there
        # (x 104 ... 231) would
        w[:, :, 120:] = 0
    eff, ref_block = (48, 40, 36), (64, 56, 64)
    out = {}
    for block, e in (((128, 128, 96), eff), (ref_block, None)):
        with M.Deconvolution(dims, 2, block, mul=mul, psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                             boundary=M.BOUNDARY_CIRCULAR, weight_norm=M.WEIGHTS_AS_GIVEN) as d:
            for v in range(2):
                d.set_view(v, imgs[v], ws[v], psfs[v])
            if e:
                d.set_effective_block_size(-1, e)
            d.prepare()
            d.run_iterations(2)
            out[block] = d.get_psi()
    big = out[(128, 128, 96)]
    assert np.isfinite(big).all()
    assert rel(big, out[ref_block]) <= 1e-5
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, ref_block, 2, mul=mul, lam=0.006, max_intensities=mx)
    assert rel(big, ref) <= 1e-4


def test_effective_block_errors():
    shape = (30, 36, 40)
    with M.Deconvolution((40, 36, 30), 2, (28, 28, 28)) as d:
        with pytest.raises(M.MvrError):
            d.set_effective_block_size(2, (10, 10, 10))
        with pytest.raises(M.MvrError):
            d.set_effective_block_size(0, (10, 0, 10))
        for v in range(2):
            d.set_view(v, np.ones(shape, np.float32), np.ones(shape, np.float32),
                       synthetic.make_psf((5, 5, 7), 1.0, 1.5, 90.0 * v))
        # 28 - 20 + 1 = 9 < 2 * 7 - 1 along z: less overlap than the doubled kernel
        d.set_effective_block_size(-1, (20, 20, 20))
        with pytest.raises(M.MvrError) as e:
            d.prepare()
        assert e.value.code == M.ERR_ARG
        d.set_effective_block_size(-1, (16, 16, 14))
        d.prepare()
        d.run_iterations(1)
        d.set_effective_block_size(-1, None)
        d.prepare()
