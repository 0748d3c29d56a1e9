"""The collocated sum factorisation of the residual and Jacobian-action
kernels, checked on the host (tests/cpp/colloc_test.cpp, g++ on the
product's quadrature header): the Gauss-point derivative matrix equals
G B^-1, and collocated interpolation and integration reproduce the direct
B/G contractions for orders 1-3."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_collocated_sum_factorisation_matches_direct(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "colloc_test"
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "cpp", "colloc_test.cpp"), "-o", str(exe)])
    p = subprocess.run([str(exe)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout[-4000:]
    assert p.stdout.strip().endswith("OK")
