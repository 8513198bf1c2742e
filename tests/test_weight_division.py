"""The weight normalisation (csrc/wdiv.h: float operations with double operations only next
to float rounding boundaries) against the reference's double formulas, bit for bit, on the
host: the same source compiled with gcc runs the division on random voxels (2-8 views,
weights in [0, 1] with zeros, ones and tiny values, sums above and below 1) and on quotients
placed on float midpoints and a double ulp either side of them; whole voxels through
mvr_wd_normalize (1-16 views, negative weights, sums at 1, hard and smooth blending, OSEM 1
and 2.5); and the fast path with its sum off by up to 2^-40 (the float pair's deviation)."""
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
    cases, bad, fallbacks, regular, regular_fallbacks, vcases, vbad, pcases, pbad = map(int, out)
    assert cases > 2_000_000 and bad == 0
    # the double division is the exception for ordinary weights (>= 1e-6)
    assert regular > 1_000_000 and regular_fallbacks <= 1e-3 * regular
    # whole voxels (1-16 views, hard and smooth, OSEM 1 and 2.5) and perturbed sums
    assert vcases > 1_000_000 and vbad == 0
    assert pcases > 50_000 and pbad == 0
