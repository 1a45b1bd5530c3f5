"""The voxelizers' vertex snapping in integer arithmetic
(voxel_cone_tracing_gb300/csrc/vct_snap.h) equals the FP64 rounding
round((g + 1) * 2^k), half to even, that the oracle uses (oracle/vct_oracle.cpp
setup of the raster and conservative rules).  Host build of the same header
the kernels include; no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_snap_fixed_matches_fp64_rounding(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "snap_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "voxel_cone_tracing_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "snap_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "100000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().startswith("0 of ")
