"""The C-ABI library builds, loads and exports exactly what include/*.h declares,
and fails loudly (no CPU fallback) where no GPU is present.  No compute calls."""
import glob
import os
import re
import subprocess

import pytest

import build_lib
import mvrgb300 as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        for m in re.finditer(r"^MVR_API\s+[\w\s\*]+?\b(\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    build_lib.build()
    return M.load()


def test_every_declared_symbol_is_exported(lib):
    declared = declared_symbols()
    assert declared == set(M.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", build_lib.LIB], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert declared <= exported
    # nothing beyond the header leaks out of the library
    assert {s for s in exported if not s.startswith("_")} == declared
    for s in declared:
        assert hasattr(lib, s)


def test_no_cpu_fallback_without_gpu(lib):
    if lib.getNumDevicesCUDA() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(M.MvrError) as e:
        M.BlockWorker((16, 16, 16))
    assert e.value.code == M.ERR_CUDA


def test_argument_errors_before_any_device_work(lib):
    with pytest.raises(M.MvrError) as e:
        M.BlockWorker((0, 16, 16))
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.BlockWorker((16, 16, 16), num_views=17)
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.BlockWorker((16, 16, 16), boundary=7)
    assert e.value.code == M.ERR_ARG


def test_psf_transformed_dims_host_geometry(lib):
    # transformPSF's output size is host arithmetic (no device work): it matches the oracle's
    # restatement for rotations, scalings and translations
    import math

    import numpy as np

    import oracle as O

    def model(ay, az, scale, t):
        a, b = math.radians(ay), math.radians(az)
        ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
        rz = np.array([[math.cos(b), -math.sin(b), 0], [math.sin(b), math.cos(b), 0], [0, 0, 1]])
        return np.hstack([rz @ ry @ np.diag(scale), np.asarray(t, dtype=np.float64).reshape(3, 1)])

    for dims in [(9, 5, 7), (31, 31, 61), (15, 11, 13)]:
        for m in [model(0, 0, (1, 1, 1), (0, 0, 0)), model(0, 90, (1, 1, 1), (3, 4, 5)),
                  model(35, 20, (1, 1, 2.5), (3.2, -1.1, 7.9)), model(-50, 0, (0.5, 0.5, 1.3), (0, 0, 0)),
                  model(45, 45, (1.5, 1, 1), (0, 0, 0))]:
            assert M.psf_transformed_dims(dims, m) == O.psf_transformed_geometry(dims, m)[0]
    with pytest.raises(M.MvrError) as e:
        M.psf_transformed_dims((5, 5, 5), np.full((3, 4), np.nan))
    assert e.value.code == M.ERR_ARG


def test_psf_and_fusion_argument_errors_before_any_device_work(lib):
    import numpy as np

    with pytest.raises(M.MvrError) as e:
        M.psf_extract(0, (8, 8, 8), [(1, 1, 1)], (5, 5, 5), 0)  # NULL image and output
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.psf_transform_normalized(0, (5, 5, 5), np.hstack([np.eye(3), np.zeros((3, 1))]), 0, (5, 5, 5))
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.psf_average([], [], True, 0)
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.psf_projection(0, (5, 5, 5), 3, True, 0)
    assert e.value.code == M.ERR_ARG
    with pytest.raises(M.MvrError) as e:
        M.fuse_group([{"img_ptr": 0, "dims": (8, 8, 8), "model": np.hstack([np.eye(3), np.zeros((3, 1))])}],
                     (0, 0, 0), (4, 4, 4), 1, 1)
    assert e.value.code == M.ERR_ARG


@pytest.mark.parametrize("dims,k,b", [((256, 256, 256), (31, 31, 61), (192, 192, 192)),
                                      ((512, 512, 256), (21, 21, 41), (192, 192, 256)),
                                      ((200, 180, 150), (9, 9, 15), (128, 128, 64)),
                                      ((37, 41, 29), (5, 7, 3), (20, 24, 16)),
                                      ((1024, 1024, 512), (41, 41, 81), (256, 256, 256))])
def test_block_grid_matches_oracle(lib, dims, k, b):
    # the host block grid of the whole-volume driver (BlockGeneratorFixedSizePrecise with the
    # doubled kernel, BlockSorter's slab dimension) against the oracle's C restatement
    import numpy as np

    import oracle as O

    kk = tuple(2 * x - 1 for x in k)
    ref = O.divide_into_blocks(dims, kk, b)
    for mr in (1, 2, 4, 1000):
        got, sd = M.block_grid(dims, k, b, mr)
        assert [tuple(map(int, g[key])) for g in got for key in ("offset", "eff_offset", "eff_size", "eff_local")] == \
               [tuple(map(int, r[key])) for r in ref for key in ("offset", "eff_offset", "eff_size", "eff_local")]
        nb = [int(np.ceil(dims[d] / (b[d] - kk[d] + 1))) for d in range(3)]
        assert sd == O.sort_dim(nb, mr)
    with pytest.raises(M.MvrError):
        M.block_grid(dims, (b[0], 3, 3), b)  # block smaller than the doubled kernel
