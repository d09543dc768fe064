"""C-ABI checks that need no GPU: the library loads and exports every symbol
that include/*.h declares, the ctypes binding covers them, and a missing
library fails loudly."""
import ctypes
import os
import re

import pytest

from conftest import ROOT, PKG

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_symbols():
    syms = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(shg_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_headers_declare_entry_points():
    syms = declared_symbols()
    for must in ["shg_context_create", "shg_ntt_forward", "shg_ntt_inverse", "shg_poly_mul",
                 "shg_poly_substitute", "shg_poly_modreduce_lsb", "shg_ct_tensor",
                 "shg_key_create", "shg_relin_apply", "shg_galois_apply",
                 "shg_bgv_mul_relin", "shg_bgv_rotate", "shg_oblivious_expand",
                 "shg_absorb_sum"]:
        assert must in syms


def test_library_exports_every_declared_symbol(sg):
    L = ctypes.CDLL(sg.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(sg):
    assert declared_symbols() <= set(sg.SIGNATURES)


def test_no_gpu_needed_for_error_paths(sg):
    """Host-side validation runs before any device work."""
    h = ctypes.c_void_p()
    qs = (ctypes.c_uint64 * 1)(1 << 40)
    code = sg.lib().shg_context_create(4, qs, 1, 65537, ctypes.byref(h))
    assert code == 3
    assert b"odd" in sg.lib().shg_last_error()
    code = sg.lib().shg_context_create(16, qs, 1, 65537, ctypes.byref(h))
    assert code == 3
    assert b"must be less than 15" in sg.lib().shg_last_error()


def test_missing_library_fails_loudly(monkeypatch):
    import importlib
    import shell_gpu
    mod = importlib.reload(shell_gpu)
    monkeypatch.setattr(mod, "LIB_PATH", os.path.join(PKG, "does-not-exist.so"))
    monkeypatch.setattr(mod, "_lib", None)
    with pytest.raises(RuntimeError, match="missing"):
        mod.lib()
    importlib.reload(shell_gpu)
