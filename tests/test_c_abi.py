"""The drop-in boundary is a C ABI: the public headers compile as strict C99
(gcc -Wall -Wextra -pedantic -Werror) and a plain C client links against
libsfx_gb300.so and runs without a GPU (tests/c/abi_client.c)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_plain_c_client(tmp_path):
    from serac_gb300 import _lib

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = tmp_path / "abi_client"
    subprocess.check_call([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(HERE, "c", "abi_client.c"), "-o", str(exe), "-L", libdir, "-lsfx_gb300",
                           "-Wl,-rpath," + libdir])
    p = subprocess.run([str(exe)], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout + p.stderr
    assert p.stdout.strip() == "OK"
