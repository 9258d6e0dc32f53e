"""The reference-dialect C++ program (tests/cxx/wrapper_usage.cpp) run on
the GPU through include/libAKAZECU/AKAZE.h: scale space, detection,
descriptors, the Matcher and MatchDescriptors, with the wrapper's own cv
subset and with the AKZ_WITH_OPENCV branch.  Every descriptor must match
itself at distance 0."""
import subprocess

import pytest

from test_library_cpu import _build_wrapper_usage

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("opencv_branch", [False, True])
@pytest.mark.parametrize("args", [[], ["--descriptor", "4"]])
def test_wrapper_program_runs(gpu_lib, tmp_path, opencv_branch, args):
    out = _build_wrapper_usage(tmp_path, opencv_branch)
    r = subprocess.run([str(out)] + args + ["--run"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "(*) Time Scale Space:" in r.stdout and "(*) Time Descriptor:" in r.stdout
    line = [s for s in r.stdout.splitlines() if "keypoints" in s][0]
    n = int(line.split()[0])
    assert n > 10 and f"{n} x 61 descriptors" in line and f"{n} self matches" in line and f"{n} x 8 match rows" in line
