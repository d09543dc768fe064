"""ctypes binding of libshellgpu.so (the C ABI declared in include/shell_gpu.h).

This is the Python-side stub a maintainer of google/shell-encryption's
tooling would write to reach the GPU path; the tests and the benchmark use it.
All polynomial buffers passed to the library are device buffers holding
uint64 Montgomery residues ([count][components][limbs][n]).
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# SHELL_GPU_LIB selects another build of the library (the SHG_DEBUG build).
LIB_PATH = os.environ.get("SHELL_GPU_LIB") or os.path.join(_HERE, "libshellgpu.so")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t

# name -> (restype, argtypes); every symbol declared in include/shell_gpu*.h.
SIGNATURES = {
    "shg_last_error": (ctypes.c_char_p, []),
    "shg_context_create": (ctypes.c_int, [ctypes.c_int, _u64p, ctypes.c_int, ctypes.c_uint64,
                                          ctypes.POINTER(_vp)]),
    "shg_context_destroy": (None, [_vp]),
    "shg_context_log_n": (ctypes.c_int, [_vp]),
    "shg_context_num_moduli": (ctypes.c_int, [_vp]),
    "shg_context_prime_info": (ctypes.c_int, [_vp, ctypes.c_int, _u64p]),
    "shg_context_ntt_tables": (ctypes.c_int, [_vp, ctypes.c_int, _u64p, _u64p]),
    "shg_context_ql_inv": (ctypes.c_int, [_vp, ctypes.c_int, _u64p]),
    "shg_ntt_forward": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_ntt_inverse": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_add": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_sub": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_neg": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_mul": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_fma": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_mul_rns_scalar": (ctypes.c_int, [_vp, _vp, _vp, _u64p, ctypes.c_int,
                                               ctypes.c_int, _vp]),
    "shg_poly_mul_integer": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_uint64, ctypes.c_int,
                                            ctypes.c_int, _vp]),
    "shg_poly_substitute": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, _vp]),
    "shg_poly_modreduce_lsb": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_uint64, _u64p,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_gadget_decompose": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _vp, _vp, ctypes.c_int,
                                            _vp]),
    "shg_poly_serialized_bytes": (_sz, [_vp, ctypes.c_int]),
    "shg_poly_serialize": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_deserialize": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_ct_tensor": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_key_create": (ctypes.c_int, [_vp, ctypes.c_int, _ip, ctypes.c_int, _u64p, _u64p,
                                      ctypes.POINTER(_vp)]),
    "shg_key_destroy": (None, [_vp]),
    "shg_key_dimension": (ctypes.c_int, [_vp]),
    "shg_key_num_limbs": (ctypes.c_int, [_vp]),
    "shg_key_log_bs": (ctypes.c_int, [_vp, _ip, ctypes.c_int]),
    "shg_key_power": (ctypes.c_int, [_vp]),
    "shg_key_context": (_vp, [_vp]),
    "shg_key_device_bytes": (_sz, [_vp]),
    "shg_relin_apply": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_relin_apply_noalloc": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_galois_apply": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_bgv_mul_relin": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_galois_precompute_pad": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_galois_apply_with_pad": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_bgv_mul_relin_multikey": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), _vp, _vp, _vp,
                                                  ctypes.c_int, _vp]),
    "shg_bgv_rotate_multikey": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), _vp, _vp, ctypes.c_int,
                                               _vp]),
    "shg_pir_expand_absorb_multikey": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.c_int, _vp,
                                                      ctypes.c_int, _vp, _vp, ctypes.c_int, _vp]),
    "shg_bgv_mul_relin_host_serialized": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int,
                                                         _vp]),
    "shg_bgv_mul_relin_host": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_bgv_rotate": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_oblivious_expand": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.c_int, _vp, _vp,
                                            ctypes.c_int, _vp]),
    "shg_pir_expand_absorb": (ctypes.c_int, [_vp, ctypes.POINTER(_vp), ctypes.c_int, _vp,
                                             ctypes.c_int, _vp, _vp, ctypes.c_int, _vp]),
    "shg_context_create_with_aux": (ctypes.c_int, [ctypes.c_int, _u64p, ctypes.c_int, _u64p,
                                                   ctypes.c_int, ctypes.c_uint64,
                                                   ctypes.POINTER(_vp)]),
    "shg_context_num_aux_moduli": (ctypes.c_int, [_vp]),
    "shg_poly_switch_rns_basis": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, _vp]),
    "shg_poly_scale_switch_rns_basis": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int,
                                                       ctypes.c_int, _vp]),
    "shg_poly_approx_switch_rns_basis": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int,
                                                        ctypes.c_int, ctypes.c_int,
                                                        ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_modreduce_msb": (ctypes.c_int, [_vp, _vp, _vp, _u64p, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, _vp]),
    "shg_poly_scale_reduce_rns_basis": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_uint64,
                                                       ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                       ctypes.c_int, _vp]),
    "shg_poly_approx_modreduce": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int,
                                                 ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, _vp]),
    "shg_bfv_mul": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "shg_bfv_absorb": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, _vp]),
    "shg_galois_key_compose": (ctypes.c_int, [_vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "shg_key_components": (ctypes.c_int, [_vp, _u64p, _u64p]),
    "shg_sample_uniform_error": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, _vp]),
    "shg_bgv_encrypt": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, _vp]),
    "shg_symmetric_encrypt": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int, _vp]),
    "shg_symmetric_decrypt": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                             _vp]),
    "shg_absorb_sum": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    # runtime plumbing (include/shell_gpu_runtime.h)
    "shg_device_count": (ctypes.c_int, [_ip]),
    "shg_set_device": (ctypes.c_int, [ctypes.c_int]),
    "shg_device_alloc": (ctypes.c_int, [_sz, ctypes.POINTER(_vp)]),
    "shg_device_free": (ctypes.c_int, [_vp]),
    "shg_host_alloc": (ctypes.c_int, [_sz, ctypes.POINTER(_vp)]),
    "shg_host_free": (ctypes.c_int, [_vp]),
    "shg_memcpy_h2d": (ctypes.c_int, [_vp, _vp, _sz, _vp]),
    "shg_memcpy_d2h": (ctypes.c_int, [_vp, _vp, _sz, _vp]),
    "shg_memcpy_d2d": (ctypes.c_int, [_vp, _vp, _sz, _vp]),
    "shg_memset_device": (ctypes.c_int, [_vp, ctypes.c_int, _sz, _vp]),
    "shg_stream_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "shg_stream_destroy": (ctypes.c_int, [_vp]),
    "shg_stream_synchronize": (ctypes.c_int, [_vp]),
    "shg_device_synchronize": (ctypes.c_int, []),
    "shg_event_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "shg_event_destroy": (ctypes.c_int, [_vp]),
    "shg_event_record": (ctypes.c_int, [_vp, _vp]),
    "shg_event_elapsed_ms": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(ctypes.c_float)]),
    "shg_graph_capture_begin": (ctypes.c_int, [_vp]),
    "shg_graph_capture_end": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "shg_graph_launch": (ctypes.c_int, [_vp, _vp]),
    "shg_graph_destroy": (ctypes.c_int, [_vp]),
    "shg_launch_count": (ctypes.c_uint64, []),
    "shg_measure_butterfly_rate": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "shg_profile_start": (ctypes.c_int, []),
    "shg_profile_stop": (ctypes.c_int, []),
    "shg_debug_status": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint)]),
    "shg_profile_query": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "shg_context_reserve": (ctypes.c_int, [_vp, _sz]),
    "shg_context_set_chunk": (ctypes.c_int, [_vp, ctypes.c_int]),
    "shg_context_set_four_step_min": (ctypes.c_int, [_vp, ctypes.c_int]),
    "shg_context_set_ks_fused": (ctypes.c_int, [_vp, ctypes.c_int]),
    "shg_context_set_ks_lanes": (ctypes.c_int, [_vp, ctypes.c_int]),
    "shg_context_set_host_pipeline": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    "shg_context_set_host_ramp": (ctypes.c_int, [_vp, ctypes.c_int]),
    "shg_context_get_tuning": (ctypes.c_int, [_vp, _ip, _ip, _ip]),
    "shg_poly_fill_uniform": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_uint64, _vp]),
    # uneven-batch executor and autotuner (include/shell_gpu_batch.h)
    "shg_batch_create": (ctypes.c_int, [ctypes.POINTER(_vp)]),
    "shg_batch_destroy": (None, [_vp]),
    "shg_batch_clear": (ctypes.c_int, [_vp]),
    "shg_batch_size": (ctypes.c_int, [_vp]),
    "shg_batch_add_mul_relin": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "shg_batch_add_rotate": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "shg_batch_add_modreduce": (ctypes.c_int, [_vp, _vp, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_uint64, _u64p]),
    "shg_batch_run": (ctypes.c_int, [_vp, _vp]),
    "shg_batch_num_groups": (ctypes.c_int, [_vp]),
    "shg_batch_autotune": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "shg_tuning_clear": (ctypes.c_int, []),
    "shg_tuning_size": (ctypes.c_int, []),
    "shg_tuning_save": (ctypes.c_int, [ctypes.c_char_p]),
    "shg_tuning_load": (ctypes.c_int, [ctypes.c_char_p]),
    "shg_tuning_lookup": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, _ip, _ip, _ip]),
}



class ServerConfig(ctypes.Structure):
    """shg_server_config (include/shell_gpu_serve.h)."""
    _fields_ = [("hbm_budget_bytes", _sz), ("max_batch", ctypes.c_int),
                ("max_wait_us", ctypes.c_int), ("num_streams", ctypes.c_int)]


class Request(ctypes.Structure):
    """shg_request (include/shell_gpu_serve.h)."""
    _fields_ = [("kind", ctypes.c_int), ("ctx", _vp), ("key", _vp),
                ("keys", ctypes.POINTER(_vp)), ("levels", ctypes.c_int), ("db", _vp),
                ("num_items", ctypes.c_int), ("in_a", _vp), ("in_b", _vp), ("out", _vp)]


class ServerStats(ctypes.Structure):
    """shg_server_stats (include/shell_gpu_serve.h)."""
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("mean_batch", ctypes.c_double), ("peak_bytes_in_flight", _sz),
                ("admission_waits", ctypes.c_uint64)]


SIGNATURES.update({
    "shg_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "shg_server_destroy": (None, [_vp]),
    "shg_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(Request),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    "shg_server_poll": (ctypes.c_int, [_vp, ctypes.c_uint64, _ip]),
    "shg_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int64]),
    "shg_server_latency": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "shg_server_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "shg_server_replay": (ctypes.c_int, [_vp, ctypes.POINTER(Request),
                                         ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_uint64)]),
})

_lib = None


class ShgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


def lib():
    """Loads libshellgpu.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: run __graft_entry__.build() to compile the CUDA library")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code != 0:
        raise ShgError(code, lib().shg_last_error().decode())


def _u64(a):
    return a.ctypes.data_as(_u64p)


class DeviceBuffer:
    """Device allocation of `nbytes` (uint64 elements)."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = _vp()
        check(lib().shg_device_alloc(max(self.nbytes, 16), ctypes.byref(p)))
        self.ptr = p.value

    @classmethod
    def from_array(cls, arr, stream=None):
        arr = np.ascontiguousarray(arr, dtype=np.uint64)
        buf = cls(arr.nbytes)
        buf.upload(arr, stream)
        return buf

    def upload(self, arr, stream=None):
        arr = np.ascontiguousarray(arr, dtype=np.uint64)
        assert arr.nbytes <= self.nbytes
        check(lib().shg_memcpy_h2d(self.ptr, arr.ctypes.data, arr.nbytes, stream))
        check(lib().shg_stream_synchronize(stream))

    def download(self, shape, stream=None):
        out = np.empty(shape, dtype=np.uint64)
        assert out.nbytes <= self.nbytes
        check(lib().shg_memcpy_d2h(out.ctypes.data, self.ptr, out.nbytes, stream))
        check(lib().shg_stream_synchronize(stream))
        return out

    def free(self):
        if self.ptr:
            lib().shg_device_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """RnsContext on the GPU (shg_context_create)."""

    def __init__(self, log_n, qs, t=65537, ps=()):
        self.log_n = log_n
        self.n = 1 << log_n
        self.qs = [int(q) for q in qs]
        self.ps = [int(p) for p in ps]
        arr = np.array(self.qs, dtype=np.uint64)
        h = _vp()
        if self.ps:
            parr = np.array(self.ps, dtype=np.uint64)
            check(lib().shg_context_create_with_aux(log_n, _u64(arr), len(self.qs), _u64(parr),
                                                    len(self.ps), int(t), ctypes.byref(h)))
        else:
            check(lib().shg_context_create(log_n, _u64(arr), len(self.qs), int(t),
                                           ctypes.byref(h)))
        self.h = h.value
        self.L = len(self.qs)
        self.K = len(self.ps)

    def close(self):
        if getattr(self, "h", None):
            lib().shg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def prime_info(self, i):
        out = np.zeros(10, np.uint64)
        check(lib().shg_context_prime_info(self.h, i, _u64(out)))
        return out

    def ntt_tables(self, i):
        f = np.zeros(self.n, np.uint64)
        v = np.zeros(self.n, np.uint64)
        check(lib().shg_context_ntt_tables(self.h, i, _u64(f), _u64(v)))
        return f, v

    def ql_inv(self, level):
        out = np.zeros(max(level, 1), np.uint64)
        check(lib().shg_context_ql_inv(self.h, level, _u64(out)))
        return out[:level]


class Key:
    """Gadget key-switching key on the GPU (shg_key_create)."""

    def __init__(self, ctx, log_bs, power, key_b, key_a):
        key_b = np.ascontiguousarray(key_b, dtype=np.uint64)
        key_a = np.ascontiguousarray(key_a, dtype=np.uint64)
        lb = np.ascontiguousarray(log_bs, dtype=np.int32)
        h = _vp()
        check(lib().shg_key_create(ctx.h, len(lb), lb.ctypes.data_as(_ip), int(power),
                                   _u64(key_b), _u64(key_a), ctypes.byref(h)))
        self.h = h.value
        self.ctx = ctx

    @property
    def dimension(self):
        return lib().shg_key_dimension(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().shg_key_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def synchronize():
    check(lib().shg_device_synchronize())
