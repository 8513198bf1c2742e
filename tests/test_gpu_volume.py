"""GPU whole-volume deconvolution (MultiViewDeconvolution{Seq,Mul} with its set-up)
against the golden fixtures and the CPU oracle.

Tolerances: PSF preparation and weights agree to float rounding (1e-6 relative);
psi after N iterations within relative L2 1e-4 of the reference-faithful oracle; the
FP64 run within 1e-9 of the oracle's FP64 run.
"""
import os

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def vol():
    return np.load(os.path.join(G, "volume_cases.npz"))


def make(vol, block, mul=False, lam=None, precision=M.PRECISION_FP32, boundary=M.BOUNDARY_REFERENCE,
         weight_norm=M.WEIGHTS_HARD, psf_type=M.PSF_OPTIMIZATION_I):
    img0 = vol["img0"]
    dims = (img0.shape[2], img0.shape[1], img0.shape[0])
    d = M.Deconvolution(dims, 2, block, mul=mul, psf_type=psf_type, psf_norm_threads=4,
                        lam=float(vol["lam"]) if lam is None else lam, boundary=boundary, precision=precision,
                        weight_norm=weight_norm)
    d.set_view(0, vol["img0"], vol["raw_w0"], vol["psf0"])
    d.set_view(1, vol["img1"], vol["raw_w1"], vol["psf1"])
    d.prepare()
    return d


def test_setup_matches_reference_semantics(vol):
    with make(vol, (28, 28, 28)) as d:
        for v in range(2):
            k1, k2 = d.kernels(v, vol["psf0"].shape)
            assert np.abs(k1 - vol[f"k1_{v}"]).max() <= 1e-6 * np.abs(vol[f"k1_{v}"]).max()
            assert np.abs(k2 - vol[f"k2_{v}"]).max() <= 1e-5 * np.abs(vol[f"k2_{v}"]).max()
            assert np.array_equal(d.weights(v), vol[f"w{v}"])
        assert np.array_equal(d.max_intensities(), vol["max"])
        assert np.allclose(d.get_psi(), vol["psi0"], rtol=1e-6)


@pytest.mark.parametrize("mul,key,block,lam", [(False, "seq", (28, 28, 28), None), (True, "mul", (28, 28, 28), None),
                                               (False, "one", (48, 44, 48), 0.0)])
def test_volume_runs_match_golden(vol, mul, key, block, lam):
    with make(vol, block, mul=mul, lam=lam) as d:
        st = d.run_iterations(2, stats=True)
        psi = d.get_psi()
    assert rel(psi, vol[key + "_psi"]) <= 1e-4
    ref = vol[key + "_stats"]
    assert np.allclose(st[:, 1], ref[:, 1], rtol=1e-3)


def test_circular_boundary_same_volume(vol):
    # the pasted effective regions do not depend on the boundary handling
    with make(vol, (28, 28, 28), boundary=M.BOUNDARY_CIRCULAR) as d:
        d.run_iterations(2)
        psi = d.get_psi()
    assert rel(psi, vol["seq_psi"]) <= 1e-4


def test_exact_batch_order_path(vol):
    # effective size 6 < k-1 = 8 along the slab axis: the deferred write-back order
    # matters, the driver follows it batch by batch
    k1 = [vol["k1_0"], vol["k1_1"]]
    k2 = [vol["k2_0"], vol["k2_1"]]
    ref, _ = O.decon_run(vol["psi0"], [vol["img0"], vol["img1"]], [vol["w0"], vol["w1"]], k1, k2, (28, 28, 22), 2,
                         lam=float(vol["lam"]), max_intensities=vol["max"])
    with make(vol, (28, 28, 22)) as d:
        d.run_iterations(2)
        psi = d.get_psi()
    assert rel(psi, ref) <= 1e-4


def test_fp64_run_against_oracle_fp64(vol):
    with make(vol, (28, 28, 28), precision=M.PRECISION_FP64) as d:
        d.run_iterations(2)
        psi64 = d.get_psi()
    # psi comes back rounded to float
    assert rel(psi64, vol["seq_psi64"]) <= 1e-7
    with make(vol, (28, 28, 28)) as d:
        d.run_iterations(2)
        psi32 = d.get_psi()
    assert rel(psi32, vol["seq_psi64"]) <= 1e-4  # FP32 error against the FP64 run


@pytest.mark.parametrize("psf_type", [0, 1, 2, 3])
def test_psf_types_against_oracle(psf_type):
    p = np.load(os.path.join(G, "psf_cases.npz"))
    raws = [p["raw0"], p["raw1"], p["raw2"]]
    dims = (24, 20, 26)
    img = np.full((26, 20, 24), 10.0, np.float32)
    with M.Deconvolution(dims, 3, (40, 40, 48), psf_type=psf_type, psf_norm_threads=4) as d:
        for v in range(3):
            d.set_view(v, img, np.ones_like(img), raws[v])
        d.prepare()
        for v in range(3):
            k1, k2 = d.kernels(v, raws[v].shape)
            r1, r2 = p[f"t{psf_type}_k1_{v}"], p[f"t{psf_type}_k2_{v}"]
            assert np.abs(k1 - r1).max() <= 1e-6 * np.abs(r1).max()
            assert np.abs(k2 - r2).max() <= 2e-5 * np.abs(r2).max()


def test_device_resident_inputs_and_update(vol):
    torch = pytest.importorskip("torch")
    img0 = torch.from_numpy(vol["img0"]).cuda()
    img1 = torch.from_numpy(vol["img1"]).cuda()
    w0 = torch.from_numpy(vol["w0"]).cuda()
    w1 = torch.from_numpy(vol["w1"]).cuda()
    dims = (40, 36, 30)
    with M.Deconvolution(dims, 2, (28, 28, 28), psf_type=M.PSF_OPTIMIZATION_I, psf_norm_threads=4,
                         lam=float(vol["lam"])) as d:
        d.set_view_device(0, img0.data_ptr(), w0.data_ptr(), vol["psf0"])
        d.set_view_device(1, img1.data_ptr(), w1.data_ptr(), vol["psf1"])
        d.prepare()
        d.run_iterations(2)
        psi = d.get_psi()
    assert rel(psi, vol["seq_psi"]) <= 1e-4


def test_errors(vol):
    with pytest.raises(M.MvrError) as e:
        M.Deconvolution((10, 10, 10), 0, (8, 8, 8))
    assert e.value.code == M.ERR_ARG
    with M.Deconvolution((40, 36, 30), 2, (28, 28, 28)) as d:
        with pytest.raises(M.MvrError) as e:
            d.prepare()  # views missing
        assert e.value.code == M.ERR_STATE
        with pytest.raises(M.MvrError) as e:
            d.run_iterations(1)
        assert e.value.code == M.ERR_STATE
    with M.Deconvolution((40, 36, 30), 2, (10, 10, 10)) as d:  # block < 2k-1
        d.set_view(0, vol["img0"], vol["raw_w0"], vol["psf0"])
        d.set_view(1, vol["img1"], vol["raw_w1"], vol["psf1"])
        with pytest.raises(M.MvrError) as e:
            d.prepare()
        assert e.value.code == M.ERR_ARG


def test_likelihood_residual(vol):
    """FP64 Poisson NLL sum_v sum_x w_v (conv1_v - img_v ln conv1_v), img_v > 0, against
    the oracle's whole-volume convolution with mirror-single extension."""
    with make(vol, (28, 28, 28)) as d:
        d.run_iterations(1)
        psi = d.get_psi()
        tot, pv = d.likelihood()
    ref_tot = 0.0
    for v in range(2):
        c1 = O.convolve(psi, vol[f"k1_{v}"], O.EXT_MIRROR_SINGLE)
        img = vol[f"img{v}"].astype(np.float64)
        w = vol[f"w{v}"].astype(np.float64)
        m = (img > 0) & (c1 > 0)
        ref = float((w[m] * (c1[m] - img[m] * np.log(c1[m]))).sum())
        assert abs(pv[v] - ref) <= 1e-5 * abs(ref)
        ref_tot += ref
    assert abs(tot - ref_tot) <= 1e-5 * abs(ref_tot)


@pytest.mark.parametrize("block,mul", [((28, 28, 28), False), ((28, 28, 22), False), ((28, 28, 28), True)])
def test_graph_replay_matches_eager_launches(vol, block, mul):
    # whole iterations captured as CUDA graphs give bit-identical psi and statistics
    # to eager launches (Jacobi path, exact batch order path, multiplicative)
    with make(vol, block, mul=mul) as d:
        d.set_graphs(False)
        st_e = d.run_iterations(5, stats=True)
        psi_e = d.get_psi()
        assert d.graphs_captured() == 0
    with make(vol, block, mul=mul) as d:
        st_g = d.run_iterations(5, stats=True)
        psi_g = d.get_psi()
        assert d.graphs_captured() >= 1
        n0 = d.launch_count()
        d.run_iterations(1, stats=True)
        assert d.launch_count() > n0  # replayed launches are counted
    assert np.array_equal(psi_g, psi_e)
    assert np.array_equal(st_g, st_e)


@pytest.mark.parametrize("mul,precision", [(False, M.PRECISION_FP32), (True, M.PRECISION_FP32),
                                           (False, M.PRECISION_FP64)])
def test_run_host_next_prefetches_the_next_inputs(vol, mul, precision):
    # mvr_decon_run_host_next: the next call's images and weights upload during this call.  A
    # sequence over two input sets (A, B = A with brighter images and other weights) gives the
    # psi of the same sequence of plain mvr_decon_run_host calls, whether the next call's arrays
    # match the prefetched ones (B after A, A after B) or not (the last call)
    a_i = [np.ascontiguousarray(vol["img0"], np.float32), np.ascontiguousarray(vol["img1"], np.float32)]
    a_w = [np.ascontiguousarray(vol["raw_w0"], np.float32), np.ascontiguousarray(vol["raw_w1"], np.float32)]
    b_i = [a * np.float32(1.25) for a in a_i]
    b_w = [np.ascontiguousarray(a_w[1]), np.ascontiguousarray(a_w[0])]
    c_i = [a * np.float32(0.8) for a in a_i]
    seq = [(a_i, a_w, b_i, b_w), (b_i, b_w, a_i, a_w), (a_i, a_w, b_i, b_w), (c_i, a_w, None, None)]
    with make(vol, (28, 28, 28), mul=mul, precision=precision) as d:
        psi0 = d.get_psi()
    ref = psi0.copy()
    with make(vol, (28, 28, 28), mul=mul, precision=precision) as d:
        refs = []
        for im, w, _, _ in seq:
            d.run_host(1, im, w, ref)
            refs.append(ref.copy())
    psi = psi0.copy()
    with make(vol, (28, 28, 28), mul=mul, precision=precision) as d:
        for (im, w, ni, nw), r in zip(seq, refs):
            d.run_host(1, im, w, psi, ni, nw)
            assert rel(psi, r) <= 1e-6
        d.run_host(2, a_i, a_w, psi, a_i, a_w)  # two iterations: the second from the graph path
        d.synchronize()
    with make(vol, (28, 28, 28), mul=mul, precision=precision) as d:
        d.run_host(2, a_i, a_w, ref)
    assert rel(psi, ref) <= 1e-6


def test_run_host_matches_device_resident_iterations(vol):
    # mvr_decon_run_host (uploads overlapped with the first view-steps) gives the same psi as
    # uploading the views and psi and running the iterations on the device
    imgs = [vol["img0"], vol["img1"]]
    raws = [vol["raw_w0"], vol["raw_w1"]]
    with make(vol, (28, 28, 28)) as d:
        psi0 = d.get_psi()
        d.run_iterations(2)
        ref = d.get_psi()
    with make(vol, (28, 28, 28)) as d:
        psi = psi0.copy()
        d.run_host(1, imgs, raws, psi)
        d.run_host(1, imgs, raws, psi)  # a second call re-uploads everything
        assert rel(psi, ref) <= 1e-6
        with make(vol, (28, 28, 28)) as d2:
            psi2 = psi0.copy()
            d2.run_host(2, imgs, raws, psi2)  # first iteration eager, the second from the graph path
        assert rel(psi2, ref) <= 1e-6
