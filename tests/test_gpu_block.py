"""GPU parity of the block iteration (through the C ABI) against the CPU oracle.

Tolerance: relative L2 <= 1e-5 per iteration for the FP32 path against the
reference-faithful oracle, <= 1e-4 after several iterations and against the FP64 run.
"""
import os

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O
import synthetic

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_ITER = 1e-5


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_case(b, kd, seed, angle=20.0, zero_frac=0.05):
    rng = np.random.default_rng(seed)
    shape = (b[2], b[1], b[0])
    k1 = synthetic.make_psf(kd, 1.0, 2.0, angle)
    k2 = O.invert_kernel(k1)
    img = rng.uniform(5, 300, shape).astype(np.float32)
    img[rng.random(shape) < zero_frac] = 0  # no data there -> quotient 1
    w = rng.uniform(0, 1, shape).astype(np.float32)
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    return psi, img, w, k1, k2


def stats_close(st, ref, psi_in, out):
    scale = float(np.abs(out.astype(np.float64) - psi_in).sum()) + 1.0
    assert abs(st.sum_change - ref[0]) <= 1e-4 * scale
    assert abs(st.max_change - ref[1]) <= 1e-4 * max(1.0, abs(ref[1]))


@pytest.mark.parametrize("b,kd,lam", [
    ((40, 36, 44), (5, 5, 9), 0.006),
    ((32, 32, 32), (7, 7, 7), 0.0),
    ((33, 27, 41), (3, 5, 7), 0.006),   # odd block sizes
    ((30, 28, 26), (4, 6, 5), 0.0),     # even kernel sizes
    ((64, 48, 40), (9, 9, 15), 0.006),
])
def test_seq_reference_boundary(b, kd, lam):
    psi, img, w, k1, k2 = make_case(b, kd, seed=sum(b))
    ref, ref_st = O.block_seq(psi, img, w, k1, k2, lam, 1e-4, 300.0)
    with M.BlockWorker(b, 1e-4, lam, 1, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        st = wk.run_iteration(0, out, img, w, 300.0)
    assert rel(out, ref) <= TOL_ITER
    stats_close(st, ref_st, psi, out)


@pytest.mark.parametrize("b,kd", [((48, 40, 60), (5, 5, 9)), ((64, 64, 64), (7, 9, 11)), ((96, 80, 72), (9, 9, 15))])
def test_seq_circular_effective_region(b, kd):
    psi, img, w, k1, k2 = make_case(b, kd, seed=7)
    ref, _ = O.block_seq(psi, img, w, k1, k2, 0.006, 1e-4, 300.0)
    with M.BlockWorker(b, 1e-4, 0.006, 1, M.BOUNDARY_CIRCULAR) as wk:
        wk.set_kernels(0, k1, k2)
        out = psi.copy()
        wk.run_iteration(0, out, img, w, 300.0)
    # effective region of a block with the doubled kernel 2k-1: k-1 voxels in from each face
    e = [k - 1 for k in kd]
    sl = (slice(e[2], b[2] - e[2]), slice(e[1], b[1] - e[1]), slice(e[0], b[0] - e[0]))
    assert rel(out[sl], ref[sl]) <= TOL_ITER


@pytest.mark.parametrize("nv", [1, 2, 3])
def test_mul_reference_boundary(nv):
    b, kd = (36, 32, 40), (5, 5, 7)
    rng = np.random.default_rng(nv)
    shape = (b[2], b[1], b[0])
    psi = rng.uniform(5, 300, shape).astype(np.float32)
    imgs = [rng.uniform(5, 300, shape).astype(np.float32) for _ in range(nv)]
    ws = [rng.uniform(0, 0.6, shape).astype(np.float32) for _ in range(nv)]
    k1s = [synthetic.make_psf(kd, 1.0, 2.0, 40.0 * v) for v in range(nv)]
    k2s = [O.invert_kernel(k) for k in k1s]
    mx = [250.0 + 10 * v for v in range(nv)]
    ref, ref_st = O.block_mul(psi, imgs, ws, k1s, k2s, 0.006, 1e-4, mx)
    with M.BlockWorker(b, 1e-4, 0.006, nv, M.BOUNDARY_REFERENCE) as wk:
        for v in range(nv):
            wk.set_kernels(v, k1s[v], k2s[v])
        out = psi.copy()
        st = wk.run_iteration_mul(out, imgs, ws, mx)
    assert rel(out, ref) <= TOL_ITER
    stats_close(st, ref_st, psi, out)


def test_golden_block_fixture():
    g = np.load(os.path.join(G, "block_cases.npz"))
    psi = g["psi"]
    b = (psi.shape[2], psi.shape[1], psi.shape[0])
    with M.BlockWorker(b, 1e-4, float(g["lam"]), 1, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, g["k1_0"], g["k2_0"])
        out = psi.copy()
        wk.run_iteration(0, out, g["img0"], g["w0"], float(g["max"][0]))
    assert rel(out, g["seq_out"]) <= TOL_ITER
    assert rel(out, g["seq_out64"]) <= 1e-4  # error against the FP64 run
    with M.BlockWorker(b, 1e-4, float(g["lam"]), 2, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, g["k1_0"], g["k2_0"])
        wk.set_kernels(1, g["k1_1"], g["k2_1"])
        out = psi.copy()
        wk.run_iteration_mul(out, [g["img0"], g["img1"]], [g["w0"], g["w1"]], g["max"])
    assert rel(out, g["mul_out"]) <= TOL_ITER
    assert rel(out, g["mul_out64"]) <= 1e-4


def test_n_iterations_against_fp32_and_fp64():
    b, kd = (48, 44, 52), (7, 7, 11)
    psi, img, w, k1, k2 = make_case(b, kd, seed=3)
    ref = psi.copy()
    ref64 = psi.astype(np.float64)
    out = psi.copy()
    with M.BlockWorker(b, 1e-4, 0.006, 1, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, k1, k2)
        for _ in range(8):
            wk.run_iteration(0, out, img, w, 300.0)
            ref, _ = O.block_seq(ref, img, w, k1, k2, 0.006, 1e-4, 300.0)
            ref64, _ = O.block_seq(ref64, img, w, k1, k2, 0.006, 1e-4, 300.0, fp64=True)
            assert rel(out, ref) <= 1e-4
    assert rel(out, ref64) <= 1e-4


def test_guards_on_gpu():
    b = (16, 16, 16)
    d = np.ones((1, 1, 1), np.float32)
    psi = np.full((16, 16, 16), 5.0, np.float32)
    psi[0] = -1.0  # psi * conv2 <= 0 -> minValue
    img = np.zeros_like(psi)  # no data: quotient 1 everywhere
    w = np.ones_like(psi)
    w[5] = 0.0  # weight 0 keeps psi
    ref, ref_st = O.block_seq(psi, img, w, d, d, 0.0, 1e-4, 10.0)
    with M.BlockWorker(b, 1e-4, 0.0, 1, M.BOUNDARY_REFERENCE) as wk:
        wk.set_kernels(0, d, d)
        out = psi.copy()
        st = wk.run_iteration(0, out, img, w, 10.0)
    assert np.array_equal(out, ref)
    assert st.max_change == pytest.approx(ref_st[1])


def test_block_at_kernel_size_and_tiny_blocks():
    for b, kd in [((5, 5, 9), (5, 5, 9)), ((2, 1, 1), (1, 1, 1)), ((8, 3, 2), (3, 3, 1))]:
        psi, img, w, k1, k2 = make_case(b, kd, seed=11, zero_frac=0.0)
        ref, _ = O.block_seq(psi, img, w, k1, k2, 0.0, 1e-4, 300.0)
        with M.BlockWorker(b, 1e-4, 0.0, 1, M.BOUNDARY_REFERENCE) as wk:
            wk.set_kernels(0, k1, k2)
            out = psi.copy()
            wk.run_iteration(0, out, img, w, 300.0)
        assert rel(out, ref) <= TOL_ITER, (b, kd)


def test_jna_convolution_in_place():
    rng = np.random.default_rng(9)
    im = rng.uniform(0, 1, (20, 24, 28)).astype(np.float32)
    k = rng.uniform(0, 1, (7, 5, 3)).astype(np.float32)
    got = M.convolution3d_fft_cuda_in_place(im, k)
    ref = O.convolve(im, k, O.EXT_ZERO)
    assert rel(got, ref) <= 1e-6


def test_device_info_and_errors():
    info = M.device_info(0)
    assert info["count"] >= 1 and info["major"] == 10 and info["mem"] > 0
    with M.BlockWorker((16, 16, 16), num_views=1) as wk:
        psi = np.ones((16, 16, 16), np.float32)
        with pytest.raises(M.MvrError) as e:
            wk.run_iteration(0, psi, psi, psi, 1.0)  # kernels not set
        assert e.value.code == M.ERR_STATE
        with pytest.raises(M.MvrError) as e:
            wk.set_kernels(3, np.ones((3, 3, 3)), np.ones((3, 3, 3)))
        assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.BlockWorker((34, 34, 34), boundary=M.BOUNDARY_CIRCULAR).set_kernels(0, np.ones((3, 3, 3)),
                                                                            np.ones((3, 3, 3)))
    assert e.value.code == M.ERR_UNSUPPORTED  # 34 = 2 * 17 is not FFT-friendly
    with pytest.raises(M.MvrError):
        M.BlockWorker((16, 16, 16), num_views=0)
