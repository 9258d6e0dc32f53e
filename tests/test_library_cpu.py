"""The C ABI library without a GPU: it builds for sm_103a, loads, exports
every symbol include/akaze_gb300.h declares, mirrors the reference's option
defaults and API shape, and reports bad arguments as status codes."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "akaze_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"AKZ_API\s+[\w\s\*]+?\b(akz_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    L = gpu_lib.load()
    declared = _declared()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(gpu_lib._lib.EXPORTS)


def test_defaults_mirror_akazeoptions(gpu_lib):
    # AKAZEConfig.h:86-111
    o = gpu_lib.AKAZEOptions()
    assert (o.omax, o.nsublevels, o.descriptor, o.descriptor_size, o.descriptor_channels) == (4, 4, 5, 0, 3)
    assert (o.descriptor_pattern_size, o.kcontrast_nbins, o.ncudaimages, o.maxkeypoints) == (10, 300, 4, 131072)
    assert (o.soffset, o.derivative_factor, o.sderivatives) == (pytest.approx(1.6), 1.5, 1.0)
    assert (o.dthreshold, o.min_dthreshold, o.kcontrast_percentile) == (
        pytest.approx(0.001), pytest.approx(1e-5), pytest.approx(0.7))
    assert o.diffusivity == gpu_lib.PM_G2
    o.setWidth(123)
    o.setHeight(45)
    assert (o.img_width, o.img_height) == (123, 45)


@pytest.mark.parametrize("field,value,status", [
    ("descriptor", 1, 6),            # SURF: not implemented (the reference prints the same)
    ("descriptor_size", 487, 1),     # more bits than the full 3-channel descriptor (AKAZE.cpp:508-509)
    ("descriptor_size", -1, 1),
    ("descriptor_channels", 4, 1),   # 1, 2 or 3 channels
    ("descriptor_channels", 0, 1),
    ("extrema_3d", 2, 1),
    ("omax", 0, 1),
    ("kcontrast_nbins", 0, 1),
    ("soffset", 0.1, 1),
    ("descriptor_pattern_size", 12, 1),
])
def test_invalid_options_are_status_codes(gpu_lib, field, value, status):
    o = gpu_lib.AKAZEOptions()
    o.setWidth(64)
    o.setHeight(64)
    setattr(o, field, value)
    h = ctypes.c_void_p()
    st = gpu_lib.load().akz_create(ctypes.byref(o), ctypes.byref(h))
    assert st == status
    assert gpu_lib.load().akz_last_error()


def test_null_and_size_errors(gpu_lib):
    L = gpu_lib.load()
    assert L.akz_options_default(None) == 1
    assert L.akz_create(None, None) == 1
    assert L.akz_feature_detection(None, None) == 1
    o = gpu_lib.AKAZEOptions()
    h = ctypes.c_void_p()
    assert L.akz_batch_create(ctypes.byref(o), 0, None, None, ctypes.byref(h)) == 1
    assert L.akz_matcher_bfmatch(None, None, 1, None, 1, 61, None) == 1


def test_python_api_mirrors_reference_binding(gpu_lib):
    # python/python_bindings.cpp:27-40 and AKAZE.h:58-143
    for name in ("Create_Nonlinear_Scale_Space", "Feature_Detection", "Compute_Descriptors", "Get_Computation_Times"):
        assert callable(getattr(gpu_lib.AKAZE, name))
    assert callable(gpu_lib.Matcher.BFMatch) and callable(gpu_lib.Matcher.bfmatch)
    assert gpu_lib.KEYPOINT_DTYPE.itemsize == 28 and gpu_lib.DMATCH_DTYPE.itemsize == 16


def _build_wrapper_usage(tmp_path, opencv_branch):
    import shutil
    import subprocess
    from pathlib import Path
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    root = Path(__file__).resolve().parent.parent
    lib_dir = root / "akaze_gb300"
    out = tmp_path / ("wrapper_usage_cv" if opencv_branch else "wrapper_usage")
    extra = ["-DAKZ_WITH_OPENCV", f"-I{root / 'tests' / 'cxx' / 'opencv_stub'}"] if opencv_branch else []
    cmd = [cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror"] + extra + [f"-I{root / 'include'}",
           str(root / "tests" / "cxx" / "wrapper_usage.cpp"), f"-L{lib_dir}", "-lakaze_gb300",
           f"-Wl,-rpath,{lib_dir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("opencv_branch", [False, True])
def test_cxx_wrapper_compiles_and_links(gpu_lib, tmp_path, opencv_branch):
    """Code in the reference demos' dialect (DESCRIPTOR_TYPE(atoi(..)),
    PM_G2, unqualified CV_32F / CV_8UC1, convertTo, operator<< on the
    options, setDefaultAKAZEOptions, Matcher, MatchDescriptors) builds
    unchanged against include/libAKAZECU/AKAZE.h, with its own cv subset and
    with AKZ_WITH_OPENCV against an OpenCV-shaped header, and links to the
    library.  Run without --run it parses and prints the options only."""
    import subprocess
    out = _build_wrapper_usage(tmp_path, opencv_branch)
    r = subprocess.run([str(out)], capture_output=True, text=True)
    assert r.returncode == 0
    lines = r.stdout.splitlines()
    assert lines[0] == "Check AKAZE options:"
    # AKAZEConfig.h:145-172: names left-aligned in 33 columns, then " =  value"
    assert lines[1] == "akaze_options.omax".ljust(33) + " =  4"
    assert "akaze_options.diffusivity".ljust(33) + " =  1" in lines
    assert "akaze_options.descriptor".ljust(33) + " =  5" in lines
    assert "akaze_options.descriptor_channels".ljust(33) + " =  3" in lines
    r = subprocess.run([str(out), "--descriptor", "4", "--diffusivity", "2", "--omax", "3"], capture_output=True, text=True)
    assert r.returncode == 0
    assert "akaze_options.descriptor".ljust(33) + " =  4" in r.stdout.splitlines()
    assert "akaze_options.diffusivity".ljust(33) + " =  2" in r.stdout.splitlines()
    assert "upright, other diffusivity" in r.stdout
    r = subprocess.run([str(out), "--descriptor", "9"], capture_output=True, text=True)  # out of range -> MLDB
    assert "akaze_options.descriptor".ljust(33) + " =  5" in r.stdout.splitlines()


@pytest.mark.parametrize("channels,size,want", [(3, 0, 61), (2, 0, 41), (1, 0, 21), (3, 256, 32), (1, 64, 8),
                                                (2, 100, 13), (3, 486, 61)])
def test_descriptor_row_bytes(gpu_lib, channels, size, want):
    """AKAZE.cpp:412-423: ceil(162 * channels / 8) bytes for the full M-LDB,
    ceil(descriptor_size / 8) for the random-bit subset."""
    o = gpu_lib.AKAZEOptions(descriptor_channels=channels, descriptor_size=size)
    assert gpu_lib.descriptor_bytes(o) == want
