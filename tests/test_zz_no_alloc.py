"""mvr_convolve_static: the block convolution for callers that cannot allocate device
memory (code inside another framework's CUDA context whose caching allocator owns the
device memory, or latency-critical paths that cannot take cudaMalloc's implicit
synchronisation).  Its scratch is one fixed device array in the library.

Checked through the C ABI on two calls in a row of different sizes (so the second call
also shows that nothing stale from the first leaks through), each against
  - the CPU oracle's linear convolution with zero extension (an independent check), and
  - the existing allocating entry point convolution3DfftCUDAInPlace,
within the relative L2 tolerance 1e-6 that the other convolution tests use.  The free
device memory reported by the driver is the same before and after a call of a size the
process has not used before.  Kept in its own file that pytest collects last.
"""
import numpy as np
import pytest

import mvrgb300 as M
import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-6
CASES = [((20, 24, 28), (7, 5, 3)), ((30, 36, 40), (9, 9, 15))]  # [z][y][x] shapes of image and kernel


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_static_scratch_convolution_matches_oracle_and_allocating_entry_point():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    stream = torch.cuda.current_stream().cuda_stream
    for img_shape, k_shape in CASES:
        img = rng.uniform(0, 1, img_shape).astype(np.float32)
        ker = rng.uniform(0, 1, k_shape).astype(np.float32)
        ref = O.convolve(img, ker, O.EXT_ZERO)  # CPU oracle, FP64
        alloc = M.convolution3d_fft_cuda_in_place(img, ker)  # allocating entry point
        d_img = torch.from_numpy(img).cuda()
        d_ker = torch.from_numpy(ker).cuda()
        d_out = torch.full(img_shape, float("nan"), dtype=torch.float32, device="cuda")
        M.convolve_static(d_img.data_ptr(), img_shape[::-1], d_ker.data_ptr(), k_shape[::-1], d_out.data_ptr(),
                          stream)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, ref) <= TOL
        assert rel(got, alloc) <= TOL


def test_static_scratch_call_allocates_no_device_memory():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream().cuda_stream
    # a first call loads the module (its static array included) on this device
    warm = torch.ones((8, 8, 8), dtype=torch.float32, device="cuda")
    warm_k = torch.ones((3, 3, 3), dtype=torch.float32, device="cuda")
    warm_out = torch.empty_like(warm)
    M.convolve_static(warm.data_ptr(), (8, 8, 8), warm_k.data_ptr(), (3, 3, 3), warm_out.data_ptr(), stream)
    torch.cuda.synchronize()
    shape, kshape = (26, 34, 46), (11, 7, 5)  # a size no other call used
    d_img = torch.from_numpy(rng.uniform(0, 1, shape).astype(np.float32)).cuda()
    d_ker = torch.from_numpy(rng.uniform(0, 1, kshape).astype(np.float32)).cuda()
    d_out = torch.empty(shape, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    M.convolve_static(d_img.data_ptr(), shape[::-1], d_ker.data_ptr(), kshape[::-1], d_out.data_ptr(), stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    ref = O.convolve(d_img.cpu().numpy(), d_ker.cpu().numpy(), O.EXT_ZERO)
    assert rel(d_out.cpu().numpy(), ref) <= TOL


def test_static_scratch_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    d_img = torch.zeros(8, dtype=torch.float32, device="cuda")
    with pytest.raises(M.MvrError) as e:
        M.convolve_static(d_img.data_ptr(), (2000, 4, 4), d_img.data_ptr(), (3, 3, 3), d_img.data_ptr())
    assert e.value.code == M.ERR_UNSUPPORTED
    assert "too large" in str(e.value)
