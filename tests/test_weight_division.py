"""The weight normalisation's division (csrc/wdiv.h: float operations with a double fallback
next to float rounding boundaries) against the reference's formula (float)((double)my / s),
bit for bit, on the host: the same source compiled with gcc runs random voxels (2-8 views,
weights in [0, 1] with zeros, ones and tiny values, sums above and below 1) and quotients
placed on float midpoints and a double ulp either side of them."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_weight_division_matches_the_double_formula(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "wdiv_check")
    subprocess.run([gcc, "-O2", "-ffp-contract=off", "-std=c99", os.path.join(HERE, "wdiv_check.c"), "-o", exe,
                    "-lm"], check=True)
    out = subprocess.run([exe, "400000"], capture_output=True, text=True, check=True).stdout.split()
    cases, bad, fallbacks, regular, regular_fallbacks = map(int, out)
    assert cases > 2_000_000 and bad == 0
    # the double division is the exception for ordinary weights (>= 1e-6)
    assert regular > 1_000_000 and regular_fallbacks <= 1e-4 * regular
