"""The kernels' division by a constant divisor (Markstein correction of the
reciprocal product) equals IEEE division for every binary32 input: an
exhaustive check over the non-negative half for both divisors in use."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_division_by_constant_is_exact_for_all_floats():
    src = os.path.join(HERE, "native", "const_div_check.c")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "const_div_check")
        subprocess.run(["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", src, "-o", exe,
                        "-lm"], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 2 and all(l.endswith("mismatches 0") for l in lines), r.stdout
    # The divisors and reciprocals the kernels hard-code.
    assert "divisor 0x3fcccccd reciprocal 0x3f200000" in lines[0]
    assert "divisor 0x3ecccccc reciprocal 0x40200001" in lines[1]
