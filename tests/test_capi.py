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
