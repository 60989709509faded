"""The reference-side binding builds into the unmodified reference driver.

capsid-souffle_gb300/dropin/forces_gb300.cpp replaces src/forces.cpp; this compiles it against
the reference's own headers and links the reference objects plus libsouffle_gb300.so into one
program (oracle/ref.mk target `dropin`).  Needs the reference tree, so it is skipped where that
is absent; running the program needs a GPU and the reference's infile layout, which the GPU
tests cover through the C ABI instead.
"""
import os
import subprocess

import pytest

from conftest import REPO

REF = os.environ.get("REF", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference tree not present")
def test_forcecalculation_binding_links_into_reference_driver():
    lib = os.path.join(REPO, "capsid-souffle_gb300", "_build", "libsouffle_gb300.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    r = subprocess.run(["make", "-f", os.path.join(REPO, "oracle", "ref.mk"), f"REF={REF}", "dropin", "-j8"],
                       cwd=REPO, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = os.path.join(REPO, "oracle", "_ref", "ref_run_gb300")
    assert os.path.exists(exe)
    nm = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # forceCalculation comes from the binding, which calls into the GPU library
    assert "forceCalculation" in nm
    assert "souffle_gpu_forces" in nm
