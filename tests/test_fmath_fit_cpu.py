"""The polynomial coefficients of akz_fmath.h are the output of the
committed fit (akaze_gb300/csrc/fit_fmath.py: Lawson's weighted minimax on
Chebyshev nodes, rounded to float32), so their provenance is reproducible."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_holds_the_fitted_coefficients():
    script = os.path.join(ROOT, "akaze_gb300", "csrc", "fit_fmath.py")
    r = subprocess.run([sys.executable, script, "--check"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["atan", "ok", "sin", "ok", "cos", "ok", "exp", "ok"]
