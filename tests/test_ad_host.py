"""The product's dual-number and material headers on the host (g++): every
forward-mode directional derivative against a central difference
(tests/cpp/ad_test.cpp, in the manner of serac's test_tensor_ad.cpp): scalar
functions, det / inv / detApIm1, the Neo-Hookean stress and first Piola flux,
and the J2 consistent tangent in elastic and plastic states."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_dual_numbers_match_central_differences(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "ad_test"
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "cpp", "ad_test.cpp"), "-o", str(exe)])
    p = subprocess.run([str(exe)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout[-4000:]
    assert p.stdout.strip().endswith("OK")
