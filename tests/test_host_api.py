"""The C++ host classes (shell-encryption_gb300/host/rlwe_gpu.h) that mirror
the reference's RnsContext / RnsPolynomial / RnsGadget / RnsBgvCiphertext /
RnsRelinKey / RnsGaloisKey / GaloisKey / GaloisKeysObliviousExpander API.

tests/cpp/host_api_test.cc exercises them against the C oracle; here it is
compiled (CPU) and run on the GPU.
"""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "shell-encryption_gb300")
SRC = os.path.join(ROOT, "tests", "cpp", "host_api_test.cc")
ERR_SRC = os.path.join(ROOT, "tests", "cpp", "error_params_test.cc")
DIGESTS = os.path.join(ROOT, "tests", "golden", "digests.json")


def _build(tmp_path, src=SRC, name="host_api_test"):
    import __graft_entry__ as ge
    if not os.path.exists(ge.HOST_LIB):
        ge.build_host()
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "host"),
           "-I", os.path.join(ROOT, "oracle"), src,
           "-L", PKG, "-lrlwe_gpu", "-lshellgpu", "-L", os.path.join(ROOT, "oracle"), "-loracle",
           f"-Wl,-rpath,{PKG}:{os.path.join(ROOT, 'oracle')}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_host_classes_compile_and_link(tmp_path, sg, oracle):
    exe = _build(tmp_path)
    assert os.path.exists(exe)


def _error_flows():
    return json.load(open(DIGESTS))["error_flow"]


@pytest.mark.parametrize("case", range(2))
def test_error_params_match_reference(tmp_path, sg, oracle, case):
    """RnsErrorParams' bounds (host-side doubles, no GPU) equal the
    reference's RnsErrorParams::Create constants bit for bit."""
    exe = _build(tmp_path, ERR_SRC, "error_params_test")
    f = _error_flows()[case]
    lb = max(f["log_bs"])
    k = sum((q.bit_length() + b - 1) // b for q, b in zip(f["qs"], f["log_bs"]))
    r = subprocess.run([exe, str(f["log_n"]), str(f["log_t"]), repr(f["sigma"]), str(lb), str(k),
                        *[str(q) for q in f["qs"]]], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [float(x) for x in r.stdout.split()]
    v = f["values"]
    assert got == [v["B_plaintext"], v["B_secretkey_encryption"], v["B_publickey_encryption"],
                   v["B_scale"], v["gadget_key_switching_bound"]]
    r = subprocess.run([exe, "0", "16", "3.19", "20", "3", "0"], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.strip() == "`log_n` must be positive."
    r = subprocess.run([exe, "10", "16", "3.19", "20", "3", "0"], capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.strip() == "`main_moduli` must not be empty."


def _error_flow_file(tmp_path, f):
    path = str(tmp_path / "error_flow.txt")
    with open(path, "w") as fh:
        fh.write(f"{f['log_n']} {f['log_t']} {f['sigma']!r} {f['e0']!r} {f['e1']!r} "
                 f"{f['scalar']} {f['power']} {len(f['qs'])}\n")
        fh.write(" ".join(str(q) for q in f["qs"]) + "\n")
        fh.write(" ".join(str(b) for b in f["log_bs"]) + "\n")
        for name, v in f["values"].items():
            fh.write(f"{name} {v!r}\n")
    return path


@pytest.mark.gpu
def test_host_classes_match_oracle_on_gpu(tmp_path, sg, oracle):
    exe = _build(tmp_path)
    # the first error-flow parameter set drives the Error() bookkeeping checks
    r = subprocess.run([exe, _error_flow_file(tmp_path, _error_flows()[0])],
                       capture_output=True, text=True, timeout=600)
    print(r.stdout[-4000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "ALL OK" in r.stdout
