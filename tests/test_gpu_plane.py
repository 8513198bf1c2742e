"""GPU parity of the plane kernels (x and y transforms fused per z-plane, used for FFT
domains Px, Py in {128, 192} with z along the tile column kernels) against the CPU
oracle, and against the row / column kernels they replace (MVR_PLANE_KERNELS=0).

Tolerances as in test_gpu_block: relative L2 <= 1e-5 per iteration against the
reference-faithful oracle; the two GPU paths agree to 1e-6.
"""
import contextlib
import os

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O
import synthetic

pytestmark = pytest.mark.gpu
TOL_ITER = 1e-5


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@contextlib.contextmanager
def plane_kernels(on):
    old = os.environ.get("MVR_PLANE_KERNELS")
    os.environ["MVR_PLANE_KERNELS"] = "1" if on else "0"
    try:
        yield
    finally:
        if old is None:
            del os.environ["MVR_PLANE_KERNELS"]
        else:
            os.environ["MVR_PLANE_KERNELS"] = old


def make_case(b, kd, seed, angle=25.0, zero_frac=0.05):
    rng = np.random.default_rng(seed)
    shape = (b[2], b[1], b[0])
    k1 = synthetic.make_psf(kd, 1.2, 2.5, angle)
    k2 = O.invert_kernel(k1)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < zero_frac] = 0
    w = rng.uniform(0, 1, shape).astype(np.float32)
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    return psi, img, w, k1, k2


def run_seq(b, boundary, psi, img, w, k1, k2, lam=0.006, on=True):
    with plane_kernels(on), M.BlockWorker(b, 1e-4, lam, 1, boundary) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        st = wk.run_iteration(0, out, img, w, 300.0)
    return out, st


@pytest.mark.parametrize("b,kd", [((128, 128, 64), (9, 9, 15)), ((192, 128, 48), (7, 9, 11)),
                                  ((128, 192, 64), (9, 7, 13)), ((192, 192, 48), (11, 11, 9))])
def test_circular_plane_kernels_effective_region(b, kd):
    psi, img, w, k1, k2 = make_case(b, kd, seed=b[0] + b[1] + b[2])
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    out, st = run_seq(b, M.BOUNDARY_CIRCULAR, psi, img, w, k1, k2)
    old, st_old = run_seq(b, M.BOUNDARY_CIRCULAR, psi, img, w, k1, k2, on=False)
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    assert rel(out[sl], ref[sl]) <= TOL_ITER
    assert rel(out, old) <= 1e-6  # the whole block, margins included
    assert st.max_change == pytest.approx(st_old.max_change, rel=1e-5, abs=1e-5)
    assert st.sum_change == pytest.approx(st_old.sum_change, rel=1e-4, abs=1e-2)


def test_reference_boundary_with_extension():
    # FFT domain 128 x 128 x 64 = block + kernel - 1: the plane kernels see the
    # mirror-single / value-1 extensions of the reference
    b, kd = (114, 114, 50), (15, 15, 15)
    psi, img, w, k1, k2 = make_case(b, kd, seed=5)
    ref, ref_st = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    out, st = run_seq(b, M.BOUNDARY_REFERENCE, psi, img, w, k1, k2)
    assert rel(out, ref) <= TOL_ITER
    scale = float(np.abs(out.astype(np.float64) - psi).sum()) + 1.0
    assert abs(st.sum_change - ref_st[0]) <= 1e-4 * scale
    assert abs(st.max_change - ref_st[1]) <= 1e-4 * max(1.0, abs(ref_st[1]))


def test_mul_plane_kernels():
    b, kd, nv = (114, 114, 56), (15, 15, 9), 2
    rng = np.random.default_rng(21)
    shape = (b[2], b[1], b[0])
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    imgs = [rng.uniform(5, 300, shape).astype(np.float32) for _ in range(nv)]
    ws = [rng.uniform(0, 0.6, shape).astype(np.float32) for _ in range(nv)]
    k1s = [synthetic.make_psf(kd, 1.0, 2.0, 50.0 * v) for v in range(nv)]
    k2s = [O.invert_kernel(k) for k in k1s]
    mx = [250.0, 270.0]
    ref, _ = O.block_mul(psi, imgs, ws, k1s, k2s, 0.006, 1e-4, mx)
    with plane_kernels(True), M.BlockWorker(b, 1e-4, 0.006, nv, M.BOUNDARY_REFERENCE) as wk:
        for v in range(nv):
            wk.set_kernels(v, k1s[v], k2s[v])
        out = psi.copy()
        wk.run_iteration_mul(out, imgs, ws, mx)
    assert rel(out, ref) <= TOL_ITER


def test_jna_convolution_plane_kernels():
    rng = np.random.default_rng(4)
    im = rng.uniform(0, 1, (50, 114, 114)).astype(np.float32)  # domain 128 x 128 x 64
    k = rng.uniform(0, 1, (15, 15, 15)).astype(np.float32)
    with plane_kernels(True):
        got = M.convolution3d_fft_cuda_in_place(im, k)
    assert rel(got, O.convolve(im, k, O.EXT_ZERO)) <= 1e-6


def test_volume_run_and_likelihood_plane_kernels():
    # a whole-volume run whose blocks take the plane kernels, against the same run on
    # the row / column kernels (likelihood included)
    dims, kd = (200, 180, 96), (9, 9, 15)
    ds = synthetic.make_dataset(dims, (0.0, 90.0), kd, n_beads=60, seed=8, side_lobes=False, weights="cosine")
    res = {}
    for on in (True, False):
        with plane_kernels(on):
            d = M.Deconvolution(dims, 2, (128, 128, 64), psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                                boundary=M.BOUNDARY_CIRCULAR, weight_norm=M.WEIGHTS_HARD)
            for v in range(2):
                d.set_view(v, ds.images[v], ds.weights[v], ds.psfs[v])
            d.prepare()
            st = d.run_iterations(3, stats=True)
            res[on] = (d.get_psi(), st, d.likelihood()[0])
            d.close()
    assert rel(res[True][0], res[False][0]) <= 1e-5
    assert np.allclose(res[True][1][:, 1], res[False][1][:, 1], rtol=1e-4, atol=1e-4)
    assert res[True][2] == pytest.approx(res[False][2], rel=1e-6)


@pytest.mark.parametrize("mul,plane,block,dims,boundary", [
    (False, True, (128, 128, 64), (200, 180, 150), M.BOUNDARY_REFERENCE),
    (True, True, (128, 128, 64), (200, 180, 150), M.BOUNDARY_REFERENCE),
    (False, False, (128, 128, 64), (200, 180, 150), M.BOUNDARY_REFERENCE),
    (False, False, (256, 256, 256), (300, 280, 270), M.BOUNDARY_REFERENCE),
    # FFT domains of the blocks themselves: the 128 x 128 and 192 x 192 plane kernels
    (False, True, (128, 128, 64), (200, 180, 150), M.BOUNDARY_CIRCULAR),
    (False, True, (192, 192, 64), (300, 280, 150), M.BOUNDARY_CIRCULAR),
    (True, True, (192, 192, 64), (300, 280, 150), M.BOUNDARY_CIRCULAR)])
def test_runs_without_statistics_write_the_same_volume(mul, plane, block, dims, boundary):
    # without statistics the plane kernels (and the row / column path's second Z pass, Y
    # inverse and update) work only on the planes and rows of each block's write region;
    # the volume they leave is bit-identical to the run that updates (and reduces) every
    # block voxel.  The plane paths also run the quotient pass only on the planes the second
    # convolution reads for the write region (the first convolution's Z pass stores zeros on
    # the others): the same volume up to float rounding of the FFTs (relative L2 1e-6), and
    # bit-identical with that band switched off (MVR_RATIO_BAND=0)
    kd = (9, 9, 15)
    ds = synthetic.make_dataset(dims, (0.0, 90.0), kd, n_beads=60, seed=9, side_lobes=False, weights="cosine")
    res = {}
    for stats, band in ((True, "1"), (False, "0"), (False, "1")):
        old = os.environ.get("MVR_RATIO_BAND")
        os.environ["MVR_RATIO_BAND"] = band
        try:
            with plane_kernels(plane):
                d = M.Deconvolution(dims, 2, block, mul=mul, psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                                    boundary=boundary, weight_norm=M.WEIGHTS_HARD)
                for v in range(2):
                    d.set_view(v, ds.images[v], ds.weights[v], ds.psfs[v])
                d.prepare()
                d.run_iterations(3, stats=stats)
                res[stats, band] = d.get_psi()
                d.close()
        finally:
            if old is None:
                del os.environ["MVR_RATIO_BAND"]
            else:
                os.environ["MVR_RATIO_BAND"] = old
    assert np.array_equal(res[True, "1"], res[False, "0"])
    assert rel(res[False, "1"], res[True, "1"]) <= 1e-6
