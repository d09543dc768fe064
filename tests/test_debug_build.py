"""The SHG_DEBUG build: kernels that check their computed indices
(substitution gathers, per-member key tables, gadget digit descriptors, limb
indices) before addressing memory, recording a failed check instead of
trapping (shg_debug_status).  It stands in for a memory checker: the parity
tests run against it, at the reference tests' small ring sizes and the larger
ones, must stay bit-exact with the oracle and leave every check clean.  The
debug library is compiled here on demand (it is not part of build()).
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SELECT = ("ntt_forward_inverse or ntt_both_kernels or substitute or tensor or gadget or "
          "relin_plain_and_fused or relin_odd_batch or galois_and_rotate or modreduce or "
          "single_modulus_galois or oblivious_expand or multikey or pir_expand_absorb")

pytestmark = pytest.mark.gpu


def test_debug_build_is_exact_and_checks_stay_clean():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    lib = ge.build_debug()
    env = dict(os.environ, SHELL_GPU_LIB=lib, SHG_DEBUG_CHECK="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-m", "gpu",
                        "-p", "no:cacheprovider", os.path.join(ROOT, "tests", "test_gpu_parity.py"),
                        "-k", SELECT], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=3000)
    print(r.stdout[-2000:])
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
