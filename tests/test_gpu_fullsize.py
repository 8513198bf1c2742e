"""Size-independent properties at the benchmark's full size (4 views, 256^3, PSF
31x31x61 Optimization-I, 192^3 blocks), where the CPU oracle is too slow to compare
against directly:

* the pasted result does not depend on the boundary handling of the block FFTs
  (circular at the block size vs the reference's padded mirror / value-1 extensions);
* it does not depend on the block size: 192^3 blocks with the reference's slab order
  give the same volume as one block covering everything (every block of a view-step
  reads the same psi when the effective size along the slab axis is >= k-1);
* the FP32 run stays within 1e-5 relative L2 of the FP64 run of the same iterations;
* the data-likelihood residual falls from iteration to iteration.
"""
import numpy as np
import pytest

import mvrgb300 as M
import synthetic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
DIMS = (256, 256, 256)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def data():
    ds = synthetic.config_256()
    imgs = [torch.from_numpy(a).cuda() for a in ds.images]
    ws = [torch.from_numpy(a).cuda() for a in ds.weights]
    return ds, imgs, ws


def run(data, block, iters, boundary=M.BOUNDARY_CIRCULAR, precision=M.PRECISION_FP32, nll=False):
    ds, imgs, ws = data
    with M.Deconvolution(DIMS, 4, block, psf_type=M.PSF_OPTIMIZATION_I, lam=0.006, boundary=boundary,
                         precision=precision, weight_norm=M.WEIGHTS_HARD) as d:
        for v in range(4):
            d.set_view_device(v, imgs[v].data_ptr(), ws[v].data_ptr(), ds.psfs[v])
        d.prepare()
        trace = []
        for _ in range(iters):
            d.run_iterations(1)
            if nll:
                trace.append(d.likelihood()[0])
        return d.get_psi(), trace


def test_boundary_and_block_size_independence(data):
    circ, nll = run(data, (192, 192, 192), 2, nll=True)
    ref, _ = run(data, (192, 192, 192), 2, boundary=M.BOUNDARY_REFERENCE)
    one, _ = run(data, (320, 320, 378), 2)
    assert rel(circ, ref) <= 1e-5
    assert rel(circ, one) <= 1e-5
    assert nll[1] < nll[0]


def test_fp32_against_fp64_run(data):
    f32, _ = run(data, (192, 192, 192), 2)
    f64, _ = run(data, (192, 192, 192), 2, precision=M.PRECISION_FP64)
    assert rel(f32, f64) <= 1e-5


def test_256_blocks_match_192_blocks(data):
    # 256^3 blocks run the row / column kernels with the persistent Z pass of 256-long
    # columns; the pasted volume equals the 192^3-block (plane kernel) run
    a, _ = run(data, (192, 192, 192), 2)
    b, _ = run(data, (256, 256, 256), 2)
    assert rel(a, b) <= 1e-5
