"""The restated MagicHat stream (pngf_gb300/csrc/hat_rng.h), which the
device-resident DBS loop draws from, against this C++ library's
std::mt19937 and std::uniform_int_distribution<int> (what MagicHat uses,
pngf-opt/magichat.hpp:53-107): engine words, bounded draws over many ranges
and whole hat passes must agree exactly."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_restated_hat_stream_matches_std(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "hat_rng_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "pngf_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "hat_rng_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")
