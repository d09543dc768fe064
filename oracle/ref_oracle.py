"""ctypes wrapper around oracle/_ref/libshellref.so — TEST INFRASTRUCTURE ONLY.

libshellref.so is google/shell-encryption's own hot-path C++ code, compiled in
place from the reference sources by oracle/ref/Makefile (only where those
sources exist; the GPU machine has only the committed golden fixtures).  It is
used to generate the golden vectors in tests/golden/ and to check the C
restatement (oracle/shell_oracle.c) against the real reference.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libshellref.so")
_U64P = ctypes.POINTER(ctypes.c_uint64)
_IP = ctypes.POINTER(ctypes.c_int)
_lib = None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_prime_tables.argtypes = [ctypes.c_uint64, ctypes.c_int, _U64P, _U64P, _U64P]
        L.ref_ntt.argtypes = [ctypes.c_uint64, ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_int]
        L.ref_rns_substitute.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_int,
                                         _U64P, _U64P]
        L.ref_rns_modreduce_lsb.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_uint64,
                                            ctypes.c_int, _U64P, _U64P]
        L.ref_bgv_mul_relin.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_uint64, _IP,
                                        _U64P, _U64P, _U64P, _U64P, ctypes.c_int, _U64P, _U64P]
        L.ref_bgv_rotate.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _IP, ctypes.c_int,
                                     _U64P, _U64P, _U64P, ctypes.c_int, _U64P]
        L.ref_oblivious_expand.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _U64P, _U64P,
                                           ctypes.c_int, _U64P]
        L.ref_serialize_vector.argtypes = [ctypes.c_uint64, _U64P, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_size_t)]
        L.ref_deserialize_vector.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint8),
                                             ctypes.c_size_t, ctypes.c_int, _U64P]
        L.ref_galois_random_pad.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _IP, ctypes.c_int,
                                            _U64P, _U64P, _U64P, _U64P, ctypes.c_int, _U64P]
        L.ref_prng_bytes.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint8)]
        L.ref_sample_uniform_error.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_char_p, _U64P, _U64P]
        L.ref_encrypt_bgv.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_int, _U64P, _U64P, ctypes.c_char_p, ctypes.c_int,
                                      _U64P]
        L.ref_switch_basis.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _U64P, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       _U64P, _U64P]
        L.ref_modreduce_msb.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, ctypes.c_int, _U64P,
                                        _U64P]
        L.ref_scale_reduce.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _U64P, ctypes.c_int,
                                       ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _U64P,
                                       ctypes.c_int, _U64P, _U64P]
        L.ref_bfv.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _U64P, ctypes.c_int,
                              ctypes.c_uint64, ctypes.c_int, ctypes.c_int, _U64P, _U64P,
                              ctypes.c_int, _U64P]
        L.ref_galois_compose.argtypes = [ctypes.c_int, _U64P, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), ctypes.c_int, _U64P,
                                         _U64P, ctypes.c_int, _U64P, _U64P, _U64P, _U64P,
                                         ctypes.POINTER(ctypes.c_int)]
        L.ref_compute_normalizer.restype = ctypes.c_uint64
        L.ref_error_flow.argtypes = [ctypes.c_int, _U64P, ctypes.c_int, _IP, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_uint64, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_double)]
        L.ref_sym_c1.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_char_p, ctypes.c_char_p, _U64P, ctypes.c_int] + \
            [_U64P] * 12 + [ctypes.POINTER(ctypes.c_double)]
        L.ref_compute_normalizer.argtypes = [ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_U64P)


def _check(code):
    if code != 0:
        raise RuntimeError(f"reference returned {code}: {lib().ref_last_error().decode()}")


def _qs(qs):
    return np.array([int(q) for q in qs], dtype=np.uint64)


def prime_tables(q, log_n):
    n = 1 << log_n
    f = np.zeros(n, np.uint64)
    i = np.zeros(n, np.uint64)
    ninv = np.zeros(1, np.uint64)
    _check(lib().ref_prime_tables(q, log_n, _p(f), _p(i), _p(ninv)))
    return f, i, int(ninv[0])


def ntt(q, log_n, data, inverse=False):
    d = np.array(data, dtype=np.uint64, copy=True).reshape(-1, 1 << log_n)
    _check(lib().ref_ntt(q, log_n, _p(d), d.shape[0], int(inverse)))
    return d.reshape(np.shape(data))


def rns_substitute(log_n, qs, poly, power):
    q = _qs(qs)
    poly = np.ascontiguousarray(poly, dtype=np.uint64)
    out = np.empty_like(poly)
    _check(lib().ref_rns_substitute(log_n, _p(q), len(q), power, _p(poly), _p(out)))
    return out


def rns_modreduce_lsb(log_n, qs, poly, t, is_ntt=True):
    q = _qs(qs)
    poly = np.ascontiguousarray(poly, dtype=np.uint64)
    out = np.empty((len(q) - 1, 1 << log_n), np.uint64)
    _check(lib().ref_rns_modreduce_lsb(log_n, _p(q), len(q), t, int(is_ntt), _p(poly), _p(out)))
    return out


def bgv_mul_relin(log_n, qs, t, log_bs, key_b, key_a, a, b):
    q = _qs(qs)
    lb = np.ascontiguousarray(log_bs, dtype=np.int32)
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    count = a.shape[0]
    L, n = len(q), 1 << log_n
    prod = np.empty((count, 3, L, n), np.uint64)
    out = np.empty((count, 2, L, n), np.uint64)
    _check(lib().ref_bgv_mul_relin(log_n, _p(q), L, t, lb.ctypes.data_as(_IP),
                                   _p(np.ascontiguousarray(key_b)),
                                   _p(np.ascontiguousarray(key_a)), _p(a), _p(b), count,
                                   _p(prod), _p(out)))
    return prod, out


def bgv_rotate(log_n, qs, log_bs, power, key_b, key_a, ct):
    q = _qs(qs)
    lb = np.ascontiguousarray(log_bs, dtype=np.int32)
    ct = np.ascontiguousarray(ct, dtype=np.uint64)
    out = np.empty_like(ct)
    _check(lib().ref_bgv_rotate(log_n, _p(q), len(q), lb.ctypes.data_as(_IP), power,
                                _p(np.ascontiguousarray(key_b)),
                                _p(np.ascontiguousarray(key_a)), _p(ct), ct.shape[0], _p(out)))
    return out


def oblivious_expand(q, log_n, log_t, levels, log_b, keys, cts):
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    cts = np.ascontiguousarray(cts, dtype=np.uint64)
    count = cts.shape[0]
    out = np.empty((count, 1 << levels, 2, 1 << log_n), np.uint64)
    _check(lib().ref_oblivious_expand(q, log_n, log_t, levels, log_b, _p(keys), _p(cts), count,
                                      _p(out)))
    return out


def compute_normalizer(k, log_t):
    return int(lib().ref_compute_normalizer(k, log_t))


def serialize_vector(q, values):
    """MontgomeryInt<uint64>::SerializeVector of the reference."""
    v = np.ascontiguousarray(values, dtype=np.uint64).reshape(-1)
    out = np.zeros(v.size * 8 + 16, np.uint8)
    nb = ctypes.c_size_t()
    _check(lib().ref_serialize_vector(q, _p(v), v.size,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                      out.size, ctypes.byref(nb)))
    return out[:nb.value].copy()


def deserialize_vector(q, data, count):
    """MontgomeryInt<uint64>::DeserializeVector of the reference."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    out = np.empty(count, np.uint64)
    _check(lib().ref_deserialize_vector(q, data.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                        data.size, count, _p(out)))
    return out


def galois_random_pad(log_n, qs, log_bs, power, key_b, key_a, cts, pad_digits):
    """RnsGaloisKey::PrecomputeRandomPad + ApplyToWithRandomPad of the reference."""
    q = _qs(qs)
    L, n = len(q), 1 << log_n
    cts = np.ascontiguousarray(cts, dtype=np.uint64)
    count = cts.shape[0]
    lb = np.ascontiguousarray(log_bs, dtype=np.int32)
    out = np.empty((count, 2, L, n), np.uint64)
    _check(lib().ref_galois_random_pad(log_n, _p(q), L, lb.ctypes.data_as(_IP), power,
                                       _p(np.ascontiguousarray(key_b, dtype=np.uint64)),
                                       _p(np.ascontiguousarray(key_a, dtype=np.uint64)),
                                       _p(cts), _p(np.ascontiguousarray(pad_digits,
                                                                         dtype=np.uint64)),
                                       count, _p(out)))
    return out


def prng_bytes(seed, count):
    """The first `count` Rand8 outputs of SingleThreadChaChaPrng::Create(seed)."""
    out = np.empty(count, np.uint8)
    _check(lib().ref_prng_bytes(bytes(seed), count,
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out


def sample_uniform_error(log_n, qs, variance, seed):
    """RnsPolynomial::SampleUniform then SampleError from one ChaCha PRNG."""
    q = _qs(qs)
    L, n = len(q), 1 << log_n
    a = np.empty((L, n), np.uint64)
    e = np.empty((L, n), np.uint64)
    _check(lib().ref_sample_uniform_error(log_n, _p(q), L, variance, bytes(seed), _p(a), _p(e)))
    return a, e


def encrypt_bgv(log_n, qs, t, variance, key, plaintexts, seeds):
    """RnsRlweSecretKey::EncryptPolynomialBgv, ciphertext c from seeds[c]."""
    q = _qs(qs)
    L, n = len(q), 1 << log_n
    plaintexts = np.ascontiguousarray(plaintexts, dtype=np.uint64)
    count = plaintexts.shape[0]
    out = np.empty((count, 2, L, n), np.uint64)
    _check(lib().ref_encrypt_bgv(log_n, _p(q), L, t, variance,
                                 _p(np.ascontiguousarray(key, dtype=np.uint64)), _p(plaintexts),
                                 b"".join(bytes(s) for s in seeds), count, _p(out)))
    return out


def switch_basis(log_n, qs, ps, level, mode, poly, is_ntt=False, balanced=False):
    """Basis conversions with the context's tables: mode 0 SwitchRnsBasis
    main -> aux, 1 aux -> main, 2 ScaleAndSwitchRnsBasis main -> aux,
    3 ApproxSwitchRnsBasis aux -> main, 4 ApproxSwitchRnsBasis main -> aux."""
    q, p = _qs(qs), _qs(ps)
    n = 1 << log_n
    n_out = len(ps) if mode in (0, 2, 4) else (len(qs) if mode == 1 else level + 1)
    poly = np.ascontiguousarray(poly, dtype=np.uint64)
    out = np.empty((n_out, n), np.uint64)
    _check(lib().ref_switch_basis(log_n, _p(q), len(q), _p(p), len(p), level, mode,
                                  int(is_ntt), int(balanced), _p(poly), _p(out)))
    return out


def modreduce_msb(log_n, qs, poly, is_ntt=True):
    q = _qs(qs)
    poly = np.ascontiguousarray(poly, dtype=np.uint64)
    out = np.empty_like(poly)
    _check(lib().ref_modreduce_msb(log_n, _p(q), len(q), int(is_ntt), _p(poly), _p(out)))
    return out[:-1]


def scale_reduce(log_n, qs, ps, t, mode, main, aux, main_ntt=True, aux_ntt=True):
    """mode 0 ScaleAndReduceRnsBasisInPlace, 1 ApproxModReduceLsb,
    2 ApproxModReduceMsb."""
    q, p = _qs(qs), _qs(ps)
    main = np.ascontiguousarray(main, dtype=np.uint64)
    aux = np.ascontiguousarray(aux, dtype=np.uint64)
    out = np.empty_like(main)
    _check(lib().ref_scale_reduce(log_n, _p(q), len(q), _p(p), len(p), t, mode,
                                  int(main_ntt), _p(main), int(aux_ntt), _p(aux), _p(out)))
    return out


def bfv_mul(log_n, qs, ps, t, a, b):
    """RnsBfvCiphertext::operator* of pairs a, b [count][2][L][n]."""
    q, p = _qs(qs), _qs(ps)
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    count = a.shape[0]
    out = np.empty((count, 3) + a.shape[2:], np.uint64)
    _check(lib().ref_bfv(log_n, _p(q), len(q), _p(p), len(p), t, 0, 2, _p(a), _p(b), count,
                         _p(out)))
    return out


def bfv_absorb(log_n, qs, ps, t, cts, pt):
    """RnsBfvCiphertext::AbsorbInPlace of cts [count][len][L][n] by pt [L][n]."""
    q, p = _qs(qs), _qs(ps)
    cts = np.ascontiguousarray(cts, dtype=np.uint64)
    pt = np.ascontiguousarray(pt, dtype=np.uint64)
    out = np.empty_like(cts)
    _check(lib().ref_bfv(log_n, _p(q), len(q), _p(p), len(p), t, 1, cts.shape[1], _p(cts),
                         _p(pt), cts.shape[0], _p(out)))
    return out


def galois_compose(log_n, qs, log_bs, power, kb, ka, power2, kb2, ka2):
    """RnsGaloisKey::Compose: (composed key_b, key_a [k][L][n], composed power)."""
    q = _qs(qs)
    lb = (ctypes.c_int * len(log_bs))(*log_bs)
    kb, ka, kb2, ka2 = (np.ascontiguousarray(x, dtype=np.uint64) for x in (kb, ka, kb2, ka2))
    ob, oa = np.empty_like(kb), np.empty_like(ka)
    pw = ctypes.c_int()
    _check(lib().ref_galois_compose(log_n, _p(q), len(q), lb, power, _p(kb), _p(ka), power2,
                                    _p(kb2), _p(ka2), _p(ob), _p(oa), ctypes.byref(pw)))
    return ob, oa, pw.value


def sym_c1(q, log_n, log_t, variance, key_seed, seeds, msgs):
    """The single-modulus symmetric flow of the reference (SymmetricRlweKey::
    Sample, Encrypt, ct + ct, ct * ct, absorb, Decrypt) on `msgs`
    [count][n] (integers in [0, t)); key from key_seed, ciphertext i from
    seeds[i] (32 bytes each).  Returns a dict of the outputs (see
    oracle/ref/ref_driver.cc ref_sym_c1)."""
    msgs = np.ascontiguousarray(msgs, dtype=np.uint64)
    count, n = msgs.shape
    half = count // 2
    o = {"s": np.empty(n, np.uint64), "pt": np.empty((count, n), np.uint64),
         "a": np.empty((count, n), np.uint64), "e": np.empty((count, n), np.uint64),
         "ct": np.empty((count, 2, n), np.uint64), "sum": np.empty((half, 2, n), np.uint64),
         "prod": np.empty((half, 3, n), np.uint64), "absorb": np.empty((half, 2, n), np.uint64),
         "dec": np.empty((count, n), np.uint64), "dec_sum": np.empty((half, n), np.uint64),
         "dec_prod": np.empty((half, n), np.uint64),
         "dec_absorb": np.empty((half, n), np.uint64)}
    err = (ctypes.c_double * 4)()
    names = ("s", "pt", "a", "e", "ct", "sum", "prod", "absorb", "dec", "dec_sum", "dec_prod",
             "dec_absorb")
    _check(lib().ref_sym_c1(q, log_n, log_t, variance, bytes(key_seed),
                            b"".join(bytes(s) for s in seeds), _p(msgs), count,
                            *[_p(o[k]) for k in names], err))
    o["err"] = np.array(list(err), np.float64)
    return o


ERROR_FLOW_FIELDS = ("B_plaintext", "B_secretkey_encryption", "B_publickey_encryption",
                     "B_scale", "gadget_key_switching_bound", "add", "sub", "absorb",
                     "absorb_scalar", "fused_absorb_add", "mul", "relin", "mod_reduce",
                     "substitute", "galois")


def error_flow(log_n, qs, log_bs, log_t, sigma, e0, e1, scalar, power):
    """Error() of the reference's RNS ciphertexts after each operation (see
    ref_error_flow in oracle/ref/ref_driver.cc); a dict keyed by
    ERROR_FLOW_FIELDS."""
    q = _qs(qs)
    lb = (ctypes.c_int * len(log_bs))(*log_bs)
    out = (ctypes.c_double * len(ERROR_FLOW_FIELDS))()
    _check(lib().ref_error_flow(log_n, _p(q), len(q), lb, log_t, sigma, e0, e1, scalar, power,
                                out))
    return dict(zip(ERROR_FLOW_FIELDS, list(out)))
