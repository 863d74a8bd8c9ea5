"""The first step's integer-pipe FP64<->FP32 conversions, FP32 error-free frame and small-rotation
quaternion update (split.cuh), checked on the host: the conversions bit-identical to the C casts,
the frame within half an ulp of 1 of the exact frame (as accurate as the FP64 frame rounded
once), the rotation within the error of the FP64 formula it replaces (both against extended
precision).  The device runs the same source with
the _rn intrinsics, so the GPU tests of the mirrors and forces cover the device side."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_split_and_frame(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "split_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "oxdna_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "native", "split_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "400000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
