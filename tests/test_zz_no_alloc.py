"""mvr_convolve_static: the block convolution for callers that cannot allocate device
memory (code inside another framework's CUDA context whose caching allocator owns the
device memory, or latency-critical paths that cannot take cudaMalloc's implicit
synchronisation).  Its scratch is one fixed device array in the library.

Checked through the C ABI against the existing allocating entry point
convolution3DfftCUDAInPlace on two calls in a row (different sizes, so the second
call also shows that nothing stale from the first leaks through), within the relative
L2 tolerance 1e-6 that the other convolution tests use.  Kept in its own file that
pytest collects last.
"""
import numpy as np
import pytest

import mvrgb300 as M

pytestmark = pytest.mark.gpu
TOL = 1e-6


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_static_scratch_convolution_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    stream = torch.cuda.current_stream().cuda_stream
    cases = [((20, 24, 28), (7, 5, 3)), ((30, 36, 40), (9, 9, 15))]  # [z][y][x] shapes
    for img_shape, k_shape in cases:
        img = rng.uniform(0, 1, img_shape).astype(np.float32)
        ker = rng.uniform(0, 1, k_shape).astype(np.float32)
        ref = M.convolution3d_fft_cuda_in_place(img, ker)  # allocating entry point
        d_img = torch.from_numpy(img).cuda()
        d_ker = torch.from_numpy(ker).cuda()
        d_out = torch.full(img_shape, float("nan"), dtype=torch.float32, device="cuda")
        M.convolve_static(d_img.data_ptr(), img_shape[::-1], d_ker.data_ptr(), k_shape[::-1], d_out.data_ptr(),
                          stream)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, ref) <= TOL


def test_static_scratch_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    d_img = torch.zeros(8, dtype=torch.float32, device="cuda")
    with pytest.raises(M.MvrError) as e:
        M.convolve_static(d_img.data_ptr(), (2000, 4, 4), d_img.data_ptr(), (3, 3, 3), d_img.data_ptr())
    assert e.value.code == M.ERR_UNSUPPORTED
    assert "too large" in str(e.value)
