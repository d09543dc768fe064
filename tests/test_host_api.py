"""The C++ host classes (shell-encryption_gb300/host/rlwe_gpu.h) that mirror
the reference's RnsContext / RnsPolynomial / RnsGadget / RnsBgvCiphertext /
RnsRelinKey / RnsGaloisKey / GaloisKey / GaloisKeysObliviousExpander API.

tests/cpp/host_api_test.cc exercises them against the C oracle; here it is
compiled (CPU) and run on the GPU.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "shell-encryption_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "host_api_test.cc")


def _build(tmp_path):
    import __graft_entry__ as ge
    if not os.path.exists(ge.HOST_LIB):
        ge.build_host()
    exe = str(tmp_path / "host_api_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "host"),
           "-I", os.path.join(ROOT, "oracle"), SRC,
           "-L", PKG, "-lrlwe_gpu", "-lshellgpu", "-L", os.path.join(ROOT, "oracle"), "-loracle",
           f"-Wl,-rpath,{PKG}:{os.path.join(ROOT, 'oracle')}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_host_classes_compile_and_link(tmp_path, sg, oracle):
    exe = _build(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_host_classes_match_oracle_on_gpu(tmp_path, sg, oracle):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "ALL OK" in r.stdout
