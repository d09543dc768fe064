"""Host logic of the uneven-batch executor that needs no GPU: the autotuner's
table (save / load / lookup, count buckets, malformed input) and argument
validation of the batch API."""
import ctypes

import pytest


@pytest.fixture
def lib(sg):
    L = sg.lib()
    sg.check(L.shg_tuning_clear())
    yield L
    L.shg_tuning_clear()


def _lookup(sg, lib, *key):
    c, f, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    code = lib.shg_tuning_lookup(*key, ctypes.byref(c), ctypes.byref(f), ctypes.byref(k))
    return code, (c.value, f.value, k.value)


def test_tuning_table_round_trip(sg, lib, tmp_path):
    src = tmp_path / "in.txt"
    # log_n L dim kind bucket chunk four_step_min ks_fused ms
    src.write_text("14 6 18 0 1024 16 14 1 28.2\n"
                   "12 3 9 1 8 4 16 0 0.31\n"
                   "\n"
                   "13 2 6 2 2 0 13 1 0.05\n")
    sg.check(lib.shg_tuning_load(str(src).encode()))
    assert lib.shg_tuning_size() == 3
    # counts map to the next power of two
    assert _lookup(sg, lib, 14, 6, 18, 0, 1000) == (0, (16, 14, 1))
    assert _lookup(sg, lib, 12, 3, 9, 1, 5) == (0, (4, 16, 0))
    assert _lookup(sg, lib, 13, 2, 6, 2, 2) == (0, (0, 13, 1))
    code, _ = _lookup(sg, lib, 14, 6, 18, 0, 2048)
    assert code == 9  # FAILED_PRECONDITION: no entry
    out = tmp_path / "out.txt"
    sg.check(lib.shg_tuning_save(str(out).encode()))
    sg.check(lib.shg_tuning_clear())
    assert lib.shg_tuning_size() == 0
    sg.check(lib.shg_tuning_load(str(out).encode()))
    assert lib.shg_tuning_size() == 3
    assert _lookup(sg, lib, 12, 3, 9, 1, 8) == (0, (4, 16, 0))


@pytest.mark.parametrize("line", ["14 6 18 0 1024 16 11 1 1.0",   # four-step min out of range
                                  "14 6 18 5 1024 16 14 1 1.0",   # unknown kind
                                  "14 6 18 0 1024 16 14 2 1.0",   # ks_fused not 0/1
                                  "14 6 18 0 1024"])              # truncated
def test_tuning_load_rejects_malformed_lines(sg, lib, tmp_path, line):
    f = tmp_path / "bad.txt"
    f.write_text("12 3 9 1 8 4 16 0 0.31\n" + line + "\n")
    code = lib.shg_tuning_load(str(f).encode())
    assert code == 3
    assert b"malformed tuning line 2" in lib.shg_last_error()
    assert lib.shg_tuning_size() == 0  # nothing of a rejected file is kept


def test_batch_api_validates_before_any_device_work(sg, lib):
    b = ctypes.c_void_p()
    sg.check(lib.shg_batch_create(ctypes.byref(b)))
    try:
        assert lib.shg_batch_size(b) == 0
        assert lib.shg_batch_num_groups(b) == 0
        assert lib.shg_batch_add_mul_relin(b, None, None, None, None, None) == 3
        assert lib.shg_batch_add_modreduce(b, None, None, None, 2, 3, 65537, None) == 3
        assert b"null context" in lib.shg_last_error()
        assert lib.shg_batch_run(b, None) == 0  # empty batch: nothing to do
        assert lib.shg_batch_autotune(b, 0, None) == 3
        sg.check(lib.shg_batch_clear(b))
    finally:
        lib.shg_batch_destroy(b)
    assert lib.shg_batch_run(None, None) == 3
