"""The contract's own binary32 transcendental functions (rfmm_math.h, used by
the galaxy seed, the control field and the display passes on the GPU and in
the oracle): their error against double-precision libm stays within a few
units in the last place (pow: exp(y ln x), whose error grows with |y ln x|
like WGSL's exp2(y log2 x) definition)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
MATH_DIR = os.path.join(os.path.dirname(HERE), "fmm-rainbow_gb300", "csrc")


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_transcendental_accuracy():
    src = os.path.join(HERE, "native", "math_accuracy.c")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "math_accuracy")
        subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-I", MATH_DIR, src, "-o", exe,
                        "-lm"], check=True)
        out = subprocess.run([exe, "1000000"], capture_output=True, text=True, check=True).stdout
    vals = dict(zip(out.split()[0::2], map(float, out.split()[1::2])))
    assert vals["sin"] < 3 and vals["cos"] < 3 and vals["exp"] < 2 and vals["log"] < 3, vals
    assert vals["atan2"] < 4, vals
    assert vals["pow"] < 64, vals  # |y ln x| up to ~40 here
