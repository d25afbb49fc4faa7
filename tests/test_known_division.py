"""The convection kernel divides by 2 dx, 2 dy, 2 dz through a precomputed
reciprocal and one remainder correction, or, for a power-of-two divisor,
by moving the exponent (see div_known in ibm_step.cu). The
reference divides; the dense step kernels are held bitwise to it, so the
replacement must equal IEEE division on every input it meets. This pins the
formula on the host (same IEEE operations as the device) over random
dividends for the divisors of the benchmark grids and random divisors."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_known_divisor_division_is_ieee(tmp_path):
    exe = tmp_path / "known_div_check"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", str(exe), os.path.join(HERE, "known_div_check.c"),
                    "-lm"], check=True)
    divisors = []
    for L, ns in ((2.5, (32, 40, 48, 64, 96, 160, 320, 640)), (0.41, (8, 12, 16, 24, 32, 64, 128))):
        divisors += [repr(2 * (L / n)) for n in ns]
    rng = np.random.default_rng(5)
    divisors += [repr(float(x)) for x in rng.uniform(1e-4, 1.0, 8)]
    # powers of two (2 dx of 2.5 / 640 is 2^-7), which take the exponent shift
    divisors += [repr(2.0 ** e) for e in (-12, -7, -1, 0, 3)]
    out = subprocess.run([str(exe), "200000", "12345"] + divisors, capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-2000:]
    assert "mismatches 0" in out.stdout
