"""The reference-side binding (tests/cpp/reference_binding_test.cc): the code a
SHELL maintainer adds, compiled against google/shell-encryption's own headers
(with the build's compatibility headers for abseil, glog and Highway) and
linked with the reference's compiled sources (oracle/_ref/libshellref.so) and
libshellgpu.so.  Real SHELL objects cross the C ABI and the GPU result is
compared with SHELL's own.  Compiling it needs the reference's sources, which
only the build container has; without a GPU the reference half runs and the
C ABI must refuse cleanly.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "shell-encryption_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "reference_binding_test.cc")
REF_LIB_DIR = os.path.join(ROOT, "oracle", "_ref")
# The reference checkout: SHELL_REFERENCE_DIR, by default the build
# container's read-only copy (absent on GPU machines: the test then skips).
REF = os.environ.get("SHELL_REFERENCE_DIR", "/root/reference")


def test_binding_compiles_against_reference_and_runs(tmp_path, sg):
    if not (os.path.isdir(os.path.join(REF, "shell_encryption")) and
            os.path.exists(os.path.join(REF_LIB_DIR, "libshellref.so"))):
        pytest.skip("reference sources / shim library absent (only the build container has them)")
    exe = str(tmp_path / "reference_binding_test")
    cmd = ["g++", "-std=gnu++17", "-O1", "-w",
           "-I", os.path.join(ROOT, "oracle", "ref", "compat"), "-I", REF,
           "-I", os.path.join(ROOT, "include"), SRC,
           "-L", REF_LIB_DIR, "-lshellref", "-L", PKG, "-lshellgpu",
           f"-Wl,-rpath,{REF_LIB_DIR}:{PKG}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout or "NO GPU" in r.stdout
