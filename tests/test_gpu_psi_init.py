"""GPU PsiInit (PsiInitAvgPrecise / PsiInitAvgApprox / PsiInitBlurredFused) against the
CPU restatements.  Tolerance: relative L2 1e-6 for the blurred fusion (double
accumulation on both sides, float storage), maxima exact, averages to 1e-9 relative."""
import os

import numpy as np
import pytest

import mvrgb300 as M
import oracle as O

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def vol():
    return np.load(os.path.join(G, "volume_cases.npz"))


def make(vol, precision=M.PRECISION_FP32):
    img0 = vol["img0"]
    dims = (img0.shape[2], img0.shape[1], img0.shape[0])
    d = M.Deconvolution(dims, 2, (28, 28, 28), psf_type=M.PSF_OPTIMIZATION_I, lam=0.006, precision=precision,
                        weight_norm=M.WEIGHTS_HARD)
    d.set_view(0, vol["img0"], vol["raw_w0"], vol["psf0"])
    d.set_view(1, vol["img1"], vol["raw_w1"], vol["psf1"])
    d.prepare()
    return d


@pytest.mark.parametrize("precision", [M.PRECISION_FP32, M.PRECISION_FP64])
@pytest.mark.parametrize("sigma", [5.0, 1.5])
def test_blurred_fused(vol, precision, sigma):
    imgs = [vol["img0"], vol["img1"]]
    with make(vol, precision) as d:
        avg = d.init_psi(M.PSI_INIT_BLURRED_FUSED, sigma)
        psi = d.get_psi()
        mx = d.max_intensities()
        ws = [d.weights(0), d.weights(1)]
        st = d.run_iterations(1, stats=True)  # the run continues from the new psi
    ref, ref_mx, ref_avg = O.psi_init_blurred_fused(imgs, ws, sigma)
    assert rel(psi, ref) <= 1e-6
    assert np.array_equal(mx, ref_mx)
    assert avg == pytest.approx(ref_avg, rel=1e-9)
    assert np.all(np.isfinite(st))


def test_avg_approx_and_back_to_precise(vol):
    imgs = [vol["img0"], vol["img1"]]
    with make(vol) as d:
        avg = d.init_psi(M.PSI_INIT_AVG_APPROX)
        psi, mx = d.get_psi(), d.max_intensities()
        ref, ref_mx, ref_avg = O.psi_init_avg_approx(imgs)
        assert avg == pytest.approx(ref_avg, rel=1e-9)
        assert np.array_equal(mx, ref_mx) and np.array_equal(psi, ref)
        d.init_psi(M.PSI_INIT_AVG_PRECISE)
        assert np.array_equal(d.max_intensities(), vol["max"])
        assert np.allclose(d.get_psi(), vol["psi0"], rtol=1e-6)
