"""The driver's parallel outfile text writer (host/text_out.h) is byte-identical to a sequential
iostream pass for the restart and movie formats (CPU only: compiles tests/native/text_out_check.cpp)."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO


@pytest.mark.parametrize("n", [1, 4095, 84000])
def test_parallel_text_writer_is_byte_identical(tmp_path, n):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "text_out_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I", os.path.join(REPO, "capsid-souffle_gb300", "host"),
                    os.path.join(REPO, "tests", "native", "text_out_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, str(n)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
