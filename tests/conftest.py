import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "shell-encryption_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# Primes used across the tests (the reference's test parameters, re-derived in
# tests/test_oracle.py).
Q45 = [35184371138561, 35184370941953, 35184370352129, 35184370155521,
       35184369893377, 35184368877569]
Q50 = [1125899904679937, 1125899903827969, 1125899903500289, 1125899903107073,
       1125899902124033, 1125899901665281, 1125899899174913, 1125899896160257,
       1125899887312897, 1125899886395393, 1125899885740033, 1125899885412353]
Q59 = 576460752303415297
Q60 = 1152921504606830593
# The largest primes below 2^58 that are 1 mod 2^16: still "small" primes (lazily
# reduced transforms), where a REDC covers only one lazy digit product.
P58 = [288230376147582977, 288230376147386369, 288230376147320833]


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def sg():
    import shell_gpu
    shell_gpu.lib()
    return shell_gpu


@pytest.fixture(autouse=True)
def _debug_checks_clean():
    """With SHG_DEBUG_CHECK set (the tests run against the SHG_DEBUG build,
    tests/test_debug_build.py), every test must leave the device-side index
    checks clean."""
    yield
    if not os.environ.get("SHG_DEBUG_CHECK"):
        return
    import ctypes
    import shell_gpu
    if shell_gpu._lib is None:
        return
    code = ctypes.c_uint(0)
    shell_gpu.check(shell_gpu.lib().shg_debug_status(ctypes.byref(code)))
    assert code.value == 0, f"a device-side index check failed (tag {code.value})"
