"""The pair plane kernels (a cluster of two CTAs per z-plane, each holding half of the rows;
the radix-2 stage of the y transform through distributed shared memory) against the CPU
oracle and against the row / column kernels, through the C ABI.

Tolerances as elsewhere: relative L2 1e-5 per iteration against the reference-faithful
oracle, 1e-6 between two GPU paths on the same inputs (float rounding only), 1e-4 after
several iterations.
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


def block_case(b, kd, seed):
    rng = np.random.default_rng(seed)
    shape = b[::-1]
    k1 = synthetic.make_psf(kd, 1.2, 2.5, 35.0)
    k2 = O.invert_kernel(k1)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < 0.05] = 0
    w = rng.uniform(0, 1, shape).astype(np.float32)
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    return psi, img, w, k1, k2


def run_block(b, boundary, psi, img, w, k1, k2, **e):
    with env(**e), M.BlockWorker(b, 1e-4, 0.006, 1, boundary) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        st = wk.run_iteration(0, out, img, w, 300.0)
    return out, st


def test_256_plane_pair_block_against_oracle_and_rows():
    # a 256 x 256 x 64 circular block: the pair kernels (MVR_PAIR_KERNELS=1) against the
    # oracle on the effective region and the row / column kernels on the whole block
    b, kd = (256, 256, 64), (15, 15, 15)
    psi, img, w, k1, k2 = block_case(b, kd, 256)
    out, st = run_block(b, M.BOUNDARY_CIRCULAR, psi, img, w, k1, k2, MVR_PAIR_KERNELS=1)
    rows, st_r = run_block(b, M.BOUNDARY_CIRCULAR, psi, img, w, k1, k2, MVR_PAIR_KERNELS=0)
    assert np.isfinite(out).all()
    assert rel(out, rows) <= 1e-6
    assert st.max_change == pytest.approx(st_r.max_change, rel=1e-5, abs=1e-5)
    assert st.sum_change == pytest.approx(st_r.sum_change, rel=1e-4, abs=1e-2)
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    assert rel(out[sl], ref[sl]) <= 1e-5


def test_256_pair_reference_boundary_whole_block():
    # block 242 x 242 x 50 with a 15^3 kernel: FFT domain 256 x 256 x 64 with the reference's
    # mirror-single / value-1 extensions, the whole block against the oracle
    b, kd = (242, 242, 50), (15, 15, 15)
    psi, img, w, k1, k2 = block_case(b, kd, 242)
    out, _ = run_block(b, M.BOUNDARY_REFERENCE, psi, img, w, k1, k2, MVR_PAIR_KERNELS=1)
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    assert rel(out, ref) <= 1e-5


def test_256_pair_mul_and_convolution():
    b, kd = (256, 256, 64), (9, 9, 11)
    rng = np.random.default_rng(7)
    shape = b[::-1]
    k1s = [synthetic.make_psf(kd, 1.0, 2.0, a) for a in (0.0, 90.0)]
    k2s = [O.invert_kernel(k) for k in k1s]
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    imgs = [rng.uniform(5, 300, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0, 1, shape).astype(np.float32) for _ in range(2)]
    outs = {}
    for on in (1, 0):
        with env(MVR_PAIR_KERNELS=on), M.BlockWorker(b, 1e-4, 0.006, 2, M.BOUNDARY_CIRCULAR) as wk:
            for v in range(2):
                wk.set_kernels(v, k1s[v], k2s[v])
            out = psi.copy()
            wk.run_iteration_mul(out, imgs, ws, [300.0, 250.0])
            outs[on] = out
    assert rel(outs[1], outs[0]) <= 1e-6
    # the reference's JNA convolution on a 256 x 256 x 64 domain (image 246 x 246 x 50, kernel
    # 11 x 11 x 15: image + kernel - 1 per axis)
    im = rng.uniform(0, 1, (50, 246, 246)).astype(np.float32)
    k = rng.uniform(0, 1, (15, 11, 11)).astype(np.float32)
    with env(MVR_PAIR_KERNELS=1):
        got = M.convolution3d_fft_cuda_in_place(im, k)
    assert rel(got, O.convolve(im, k, O.EXT_ZERO)) <= 1e-6


@pytest.mark.parametrize("block,dims", [((192, 192, 64), (260, 250, 90)), ((256, 256, 64), (300, 290, 80))])
def test_forced_pair_schedule_matches_rows_and_oracle(block, dims):
    rng = np.random.default_rng(block[0])
    shape = dims[::-1]
    psfs = [synthetic.make_psf((9, 9, 15), 1.2, 2.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 200, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    out = {}
    for code in (M.SCHED_PAIR, M.SCHED_PAIR | M.SCHED_ZPIPE, M.SCHED_ROWS):
        with M.Deconvolution(dims, 2, block, psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                             boundary=M.BOUNDARY_CIRCULAR, weight_norm=M.WEIGHTS_AS_GIVEN) as d:
            for v in range(2):
                d.set_view(v, imgs[v], ws[v], psfs[v])
            d.set_schedule(code)
            d.prepare()
            assert d.schedule(0) == code
            st = d.run_iterations(2, stats=True)
            out[code] = (d.get_psi(), st)
    base, st_b = out[M.SCHED_ROWS]
    for code in (M.SCHED_PAIR, M.SCHED_PAIR | M.SCHED_ZPIPE):
        psi, st = out[code]
        assert rel(psi, base) <= 1e-6
        assert np.allclose(st[:, 1], st_b[:, 1], rtol=1e-4)
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, block, 2, lam=0.006, max_intensities=mx)
    assert rel(out[M.SCHED_PAIR][0], ref) <= 1e-4
