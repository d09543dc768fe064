"""ctypes wrapper around the CPU oracle (liboracle.so) — TEST INFRASTRUCTURE ONLY.

The oracle restates google/shell-encryption's CPU algorithms for the RLWE
polynomial hot path in plain C (oracle/shell_oracle.c).  Only the test suite,
the smoke check and the benchmark's CPU-baseline leg import this module, as
the checker or as the timed CPU baseline; the GPU library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

U64P = ctypes.POINTER(ctypes.c_uint64)
INTP = ctypes.POINTER(ctypes.c_int)


def build():
    """Compiles liboracle.so from oracle/shell_oracle.c (gcc via make)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        sig = {
            "so_prime_create": (vp, [ctypes.c_uint64, ctypes.c_int]),
            "so_prime_destroy": (None, [vp]),
            "so_prime_info": (None, [vp, U64P]),
            "so_prime_tables": (None, [vp, U64P, U64P]),
            "so_import": (None, [vp, U64P, U64P, ctypes.c_size_t]),
            "so_export": (None, [vp, U64P, U64P, ctypes.c_size_t]),
            "so_add": (None, [vp, U64P, U64P, U64P, ctypes.c_size_t]),
            "so_sub": (None, [vp, U64P, U64P, U64P, ctypes.c_size_t]),
            "so_neg": (None, [vp, U64P, U64P, ctypes.c_size_t]),
            "so_mul": (None, [vp, U64P, U64P, U64P, ctypes.c_size_t]),
            "so_fma": (None, [vp, U64P, U64P, U64P, ctypes.c_size_t]),
            "so_mul_scalar": (None, [vp, U64P, ctypes.c_uint64, U64P, ctypes.c_size_t]),
            "so_ntt_fwd": (None, [vp, U64P]),
            "so_ntt_inv": (None, [vp, U64P]),
            "so_substitute": (ctypes.c_int, [vp, ctypes.c_int, U64P, U64P]),
            "so_rns_create": (vp, [ctypes.c_int, U64P, ctypes.c_int]),
            "so_rns_destroy": (None, [vp]),
            "so_rns_prime": (vp, [vp, ctypes.c_int]),
            "so_rns_ql_inv": (None, [vp, ctypes.c_int, U64P]),
            "so_rns_complements": (None, [vp, ctypes.c_int, U64P, U64P]),
            "so_rns_gadget_dim": (ctypes.c_int, [vp, ctypes.c_int, INTP]),
            "so_rns_gadget_vector": (None, [vp, ctypes.c_int, INTP, U64P]),
            "so_rns_ntt_fwd": (None, [vp, U64P, ctypes.c_int]),
            "so_rns_ntt_inv": (None, [vp, U64P, ctypes.c_int]),
            "so_rns_substitute": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, U64P, U64P]),
            "so_rns_decompose": (None, [vp, ctypes.c_int, INTP, U64P, U64P]),
            "so_rns_tensor": (None, [vp, ctypes.c_int, U64P, U64P, U64P]),
            "so_rns_relin": (None, [vp, ctypes.c_int, INTP, U64P, U64P, U64P, U64P]),
            "so_rns_galois": (None, [vp, ctypes.c_int, INTP, U64P, U64P, U64P, U64P]),
            "so_rns_modreduce_lsb": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_uint64,
                                                    ctypes.c_int, U64P, U64P]),
            "so_rns_mul_relin_batch": (None, [vp, ctypes.c_int, INTP, U64P, U64P, U64P,
                                              U64P, U64P, ctypes.c_int, ctypes.c_int]),
            "so_gadget_size": (ctypes.c_int, [vp, ctypes.c_int]),
            "so_keyswitch_part": (None, [vp, ctypes.c_int, ctypes.c_int, U64P, U64P, U64P,
                                         U64P, U64P]),
            "so_galois_apply": (None, [vp, ctypes.c_int, ctypes.c_int, U64P, U64P, U64P, U64P]),
            "so_oblivious_expand": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, U64P,
                                                   U64P, U64P]),
            "so_absorb_sum": (None, [vp, ctypes.c_int, U64P, U64P, U64P]),
            "so_serialize_vector": (ctypes.c_size_t, [vp, U64P, ctypes.c_size_t,
                                                      ctypes.POINTER(ctypes.c_uint8)]),
            "so_deserialize_vector": (None, [vp, ctypes.POINTER(ctypes.c_uint8),
                                             ctypes.c_size_t, U64P]),
            "so_rns_galois_pad": (None, [vp, ctypes.c_int, ctypes.c_int, U64P, U64P, U64P, U64P,
                                         U64P]),
            "so_rns_switch_basis": (None, [vp, INTP, ctypes.c_int, INTP, ctypes.c_int, U64P,
                                           U64P]),
            "so_rns_scale_switch_basis": (None, [vp, INTP, ctypes.c_int, INTP, ctypes.c_int,
                                                 U64P, U64P]),
            "so_rns_approx_switch_basis": (None, [vp, INTP, ctypes.c_int, INTP, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_int, U64P, U64P]),
            "so_rns_modreduce_msb": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, U64P,
                                                    U64P]),
            "so_rns_scale_reduce": (None, [vp, ctypes.c_int, INTP, ctypes.c_int, ctypes.c_uint64,
                                           ctypes.c_int, U64P, ctypes.c_int, U64P, U64P]),
            "so_rns_approx_modreduce_lsb": (None, [vp, ctypes.c_int, INTP, ctypes.c_int,
                                                   ctypes.c_uint64, ctypes.c_int, U64P,
                                                   ctypes.c_int, U64P, U64P]),
            "so_rns_approx_modreduce_msb": (None, [vp, ctypes.c_int, INTP, ctypes.c_int,
                                                   ctypes.c_int, U64P, ctypes.c_int, U64P,
                                                   U64P]),
            "so_bfv_mul": (None, [vp, ctypes.c_int, INTP, ctypes.c_int, ctypes.c_uint64, U64P,
                                  U64P, U64P]),
            "so_bfv_absorb": (None, [vp, ctypes.c_int, INTP, ctypes.c_int, ctypes.c_uint64,
                                     ctypes.c_int, U64P, U64P, U64P]),
            "so_chacha20_block": (None, [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_char_p,
                                         ctypes.POINTER(ctypes.c_uint8)]),
            "so_prng_bytes": (None, [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_uint8)]),
            "so_rns_sample_uniform_error": (None, [vp, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_char_p, U64P, U64P]),
            "so_rns_encrypt_bgv": (None, [vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_int, U64P,
                                          U64P, ctypes.c_char_p, U64P]),
            "so_sym_encrypt": (None, [vp, ctypes.c_uint64, U64P, U64P, U64P, U64P, U64P]),
            "so_sym_decrypt": (None, [vp, ctypes.c_uint64, U64P, U64P, ctypes.c_int, U64P]),
            "so_sym_key_sample": (None, [vp, ctypes.c_int, ctypes.c_char_p, U64P]),
            "so_sym_encrypt_prng": (None, [vp, ctypes.c_uint64, ctypes.c_int, U64P, U64P,
                                           ctypes.c_char_p, U64P]),
            "so_compute_normalizer": (ctypes.c_uint64, [ctypes.c_int, ctypes.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(U64P)


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(INTP)


class Prime:
    """One prime q at ring degree 2^log_n (MontgomeryIntParams + NttParameters)."""

    def __init__(self, q, log_n, _handle=None, _owner=None):
        self.q = int(q)
        self.log_n = log_n
        self.n = 1 << log_n
        if _handle is None:
            h = lib().so_prime_create(ctypes.c_uint64(self.q), log_n)
            if not h:
                raise ValueError("invalid prime / log_n")
            self._h = h
            self._own = True
        else:
            self._h = _handle
            self._own = False
            self._owner = _owner

    def __del__(self):
        if getattr(self, "_own", False) and _lib is not None:
            _lib.so_prime_destroy(self._h)

    def info(self):
        out = np.zeros(10, np.uint64)
        lib().so_prime_info(self._h, _p(out))
        keys = ["q", "log_q", "inv_modulus", "r_mod_q", "r_mod_q_barrett", "inv_r",
                "inv_r_barrett", "barrett_num", "psi", "n_inv"]
        return {k: int(v) for k, v in zip(keys, out)}

    def tables(self):
        f = np.zeros(self.n, np.uint64)
        i = np.zeros(self.n, np.uint64)
        lib().so_prime_tables(self._h, _p(f), _p(i))
        return f, i

    def _un(self, fn, a):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        out = np.empty_like(a)
        fn(self._h, _p(a), _p(out), a.size)
        return out

    def _bin(self, fn, a, b):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        out = np.empty_like(a)
        fn(self._h, _p(a), _p(b), _p(out), a.size)
        return out

    def import_(self, a):
        return self._un(lib().so_import, a)

    def export(self, a):
        return self._un(lib().so_export, a)

    def add(self, a, b):
        return self._bin(lib().so_add, a, b)

    def sub(self, a, b):
        return self._bin(lib().so_sub, a, b)

    def neg(self, a):
        return self._un(lib().so_neg, a)

    def mul(self, a, b):
        return self._bin(lib().so_mul, a, b)

    def fma(self, acc, a, b):
        acc = np.array(acc, dtype=np.uint64, copy=True)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        lib().so_fma(self._h, _p(acc), _p(a), _p(b), acc.size)
        return acc

    def mul_scalar(self, a, s):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        out = np.empty_like(a)
        lib().so_mul_scalar(self._h, _p(a), ctypes.c_uint64(int(s)), _p(out), a.size)
        return out

    def ntt_fwd(self, a):
        a = np.array(a, dtype=np.uint64, copy=True)
        assert a.size == self.n
        lib().so_ntt_fwd(self._h, _p(a))
        return a

    def ntt_inv(self, a):
        a = np.array(a, dtype=np.uint64, copy=True)
        assert a.size == self.n
        lib().so_ntt_inv(self._h, _p(a))
        return a

    def substitute(self, a, power):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        out = np.empty_like(a)
        st = lib().so_substitute(self._h, power, _p(a), _p(out))
        if st:
            raise ValueError("Substitution power must be a non-negative odd integer less than 2*n.")
        return out

    def gadget_size(self, log_b):
        return lib().so_gadget_size(self._h, log_b)

    def keyswitch_part(self, log_b, c, k0, k1):
        dim = self.gadget_size(log_b)
        c = np.ascontiguousarray(c, dtype=np.uint64)
        k0 = np.ascontiguousarray(k0, dtype=np.uint64)
        k1 = np.ascontiguousarray(k1, dtype=np.uint64)
        o0 = np.empty(self.n, np.uint64)
        o1 = np.empty(self.n, np.uint64)
        lib().so_keyswitch_part(self._h, log_b, dim, _p(c), _p(k0), _p(k1), _p(o0), _p(o1))
        return o0, o1

    def galois_apply(self, log_b, ct, k0, k1):
        dim = self.gadget_size(log_b)
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        k0 = np.ascontiguousarray(k0, dtype=np.uint64)
        k1 = np.ascontiguousarray(k1, dtype=np.uint64)
        out = np.empty((2, self.n), np.uint64)
        lib().so_galois_apply(self._h, log_b, dim, _p(ct), _p(k0), _p(k1), _p(out))
        return out

    def oblivious_expand(self, levels, log_b, keys, ct):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        out = np.empty((1 << levels, 2, self.n), np.uint64)
        st = lib().so_oblivious_expand(self._h, levels, log_b, _p(keys), _p(ct), _p(out))
        if st:
            raise ValueError("bad levels")
        return out

    def serialize(self, v):
        v = np.ascontiguousarray(v, dtype=np.uint64).reshape(-1)
        out = np.zeros((v.size * self.info()["log_q"] + 7) // 8, np.uint8)
        nb = lib().so_serialize_vector(self._h, _p(v), v.size,
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return out[:nb]

    def deserialize(self, data, count):
        data = np.ascontiguousarray(data, dtype=np.uint8)
        out = np.empty(count, np.uint64)
        lib().so_deserialize_vector(self._h, data.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                    count, _p(out))
        return out

    def sym_encrypt(self, t, s, a, e, m):
        """(c0, c1) = (NTT(e) * t + m + a * s, -a); s, a, m NTT form, e coefficients."""
        arrs = [np.ascontiguousarray(x, dtype=np.uint64) for x in (s, a, e, m)]
        out = np.empty((2, self.n), np.uint64)
        lib().so_sym_encrypt(self._h, ctypes.c_uint64(int(t)), *[_p(x) for x in arrs], _p(out))
        return out

    def sym_key_sample(self, variance, seed):
        """SymmetricRlweKey::Sample from the ChaCha PRNG of the 32-byte seed."""
        out = np.empty(self.n, np.uint64)
        lib().so_sym_key_sample(self._h, variance, bytes(seed), _p(out))
        return out

    def sym_encrypt_prng(self, t, variance, s, m, seed):
        """rlwe::Encrypt with the ChaCha PRNG of the 32-byte seed."""
        s = np.ascontiguousarray(s, dtype=np.uint64)
        m = np.ascontiguousarray(m, dtype=np.uint64)
        out = np.empty((2, self.n), np.uint64)
        lib().so_sym_encrypt_prng(self._h, ctypes.c_uint64(int(t)), variance, _p(s), _p(m),
                                  bytes(seed), _p(out))
        return out

    def sym_decrypt(self, t, s, ct):
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        s = np.ascontiguousarray(s, dtype=np.uint64)
        out = np.empty(self.n, np.uint64)
        lib().so_sym_decrypt(self._h, ctypes.c_uint64(int(t)), _p(s), _p(ct), ct.shape[0],
                             _p(out))
        return out

    def absorb_sum(self, cts, db):
        cts = np.ascontiguousarray(cts, dtype=np.uint64)
        db = np.ascontiguousarray(db, dtype=np.uint64)
        out = np.empty((2, self.n), np.uint64)
        lib().so_absorb_sum(self._h, cts.shape[0], _p(cts), _p(db), _p(out))
        return out


class Rns:
    """RNS context over primes qs at ring degree 2^log_n (RnsContext)."""

    def __init__(self, log_n, qs):
        self.log_n = log_n
        self.n = 1 << log_n
        self.qs = [int(q) for q in qs]
        self.L = len(qs)
        arr = np.array(self.qs, dtype=np.uint64)
        h = lib().so_rns_create(log_n, _p(arr), self.L)
        if not h:
            raise ValueError("invalid RNS moduli")
        self._h = h
        self.primes = [Prime(q, log_n, _handle=lib().so_rns_prime(h, i), _owner=self)
                       for i, q in enumerate(self.qs)]

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.so_rns_destroy(self._h)
            self._h = None

    def ql_inv(self, level):
        out = np.zeros(max(level, 1), np.uint64)
        lib().so_rns_ql_inv(self._h, level, _p(out))
        return out[:level]

    def complements(self, level):
        a = np.zeros(level + 1, np.uint64)
        b = np.zeros(level + 1, np.uint64)
        lib().so_rns_complements(self._h, level, _p(a), _p(b))
        return a, b

    def gadget_dim(self, log_bs):
        lb, p = _ip(log_bs)
        return lib().so_rns_gadget_dim(self._h, len(lb), p)

    def gadget_vector(self, log_bs):
        lb, p = _ip(log_bs)
        k = lib().so_rns_gadget_dim(self._h, len(lb), p)
        g = np.zeros((k, len(lb)), np.uint64)
        lib().so_rns_gadget_vector(self._h, len(lb), p, _p(g))
        return g

    def ntt_fwd(self, poly):
        poly = np.array(poly, dtype=np.uint64, copy=True)
        lib().so_rns_ntt_fwd(self._h, _p(poly), poly.shape[-2])
        return poly

    def ntt_inv(self, poly):
        poly = np.array(poly, dtype=np.uint64, copy=True)
        lib().so_rns_ntt_inv(self._h, _p(poly), poly.shape[-2])
        return poly

    def substitute(self, poly, power):
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        out = np.empty_like(poly)
        st = lib().so_rns_substitute(self._h, poly.shape[0], power, _p(poly), _p(out))
        if st:
            raise ValueError("Substitution power must be a non-negative odd integer less than 2*n.")
        return out

    def decompose(self, poly, log_bs):
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        L = poly.shape[0]
        lb, p = _ip(log_bs)
        k = lib().so_rns_gadget_dim(self._h, L, p)
        out = np.empty((k, L, self.n), np.uint64)
        lib().so_rns_decompose(self._h, L, p, _p(poly), _p(out))
        return out

    def tensor(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        L = a.shape[1]
        out = np.empty((3, L, self.n), np.uint64)
        lib().so_rns_tensor(self._h, L, _p(a), _p(b), _p(out))
        return out

    def relin(self, ct, key_b, key_a, log_bs):
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        L = ct.shape[1]
        lb, p = _ip(log_bs)
        out = np.empty((2, L, self.n), np.uint64)
        lib().so_rns_relin(self._h, L, p, _p(ct), _p(np.ascontiguousarray(key_b)),
                           _p(np.ascontiguousarray(key_a)), _p(out))
        return out

    def galois(self, ct, key_b, key_a, log_bs):
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        L = ct.shape[1]
        lb, p = _ip(log_bs)
        out = np.empty((2, L, self.n), np.uint64)
        lib().so_rns_galois(self._h, L, p, _p(ct), _p(np.ascontiguousarray(key_b)),
                            _p(np.ascontiguousarray(key_a)), _p(out))
        return out

    def galois_pad(self, ct, pad, key_b, key_a):
        """RnsGaloisKey::PrecomputeRandomPad + ApplyToWithRandomPad."""
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        pad = np.ascontiguousarray(pad, dtype=np.uint64)
        L = ct.shape[1]
        out = np.empty_like(ct)
        lib().so_rns_galois_pad(self._h, L, pad.shape[0], _p(ct), _p(pad),
                                _p(np.ascontiguousarray(key_b, dtype=np.uint64)),
                                _p(np.ascontiguousarray(key_a, dtype=np.uint64)), _p(out))
        return out

    def sample_uniform_error(self, L, variance, seed):
        """SampleUniform then SampleError from the ChaCha PRNG of `seed`."""
        a = np.empty((L, self.n), np.uint64)
        e = np.empty((L, self.n), np.uint64)
        lib().so_rns_sample_uniform_error(self._h, L, variance, bytes(seed), _p(a), _p(e))
        return a, e

    def encrypt_bgv(self, t, variance, key, m, seed):
        """RnsRlweSecretKey::EncryptPolynomialBgv with the PRNG of `seed`."""
        key = np.ascontiguousarray(key, dtype=np.uint64)
        m = np.ascontiguousarray(m, dtype=np.uint64)
        L = m.shape[0]
        out = np.empty((2, L, self.n), np.uint64)
        lib().so_rns_encrypt_bgv(self._h, L, ctypes.c_uint64(int(t)), variance, _p(key), _p(m),
                                 bytes(seed), _p(out))
        return out

    # ---- basis conversion and BFV: the context's primes are the main primes
    # followed by the auxiliary ones; src / dst / aux are prime indices. ----

    def switch_basis(self, src, dst, poly, scale=False):
        """SwitchRnsBasis (scale=False) or ScaleAndSwitchRnsBasis (scale=True)
        of a coefficient-form polynomial [len(src)][n] -> [len(dst)][n]."""
        s, sp = _ip(src)
        d, dp = _ip(dst)
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        out = np.empty((len(d), self.n), np.uint64)
        fn = lib().so_rns_scale_switch_basis if scale else lib().so_rns_switch_basis
        fn(self._h, sp, len(s), dp, len(d), _p(poly), _p(out))
        return out

    def approx_switch_basis(self, src, dst, poly, is_ntt, balanced):
        s, sp = _ip(src)
        d, dp = _ip(dst)
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        out = np.empty((len(d), self.n), np.uint64)
        lib().so_rns_approx_switch_basis(self._h, sp, len(s), dp, len(d), int(is_ntt),
                                         int(balanced), _p(poly), _p(out))
        return out

    def modreduce_msb(self, poly, is_ntt=True):
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        L = poly.shape[0]
        out = np.empty((L - 1, self.n), np.uint64)
        if lib().so_rns_modreduce_msb(self._h, L, int(is_ntt), _p(poly), _p(out)):
            raise ValueError("ModReduceMsb needs two or more limbs")
        return out

    def scale_reduce(self, aux, t, main, aux_poly, main_ntt=True, aux_ntt=True, mode=0):
        """mode 0 ScaleAndReduceRnsBasisInPlace, 1 ApproxModReduceLsb,
        2 ApproxModReduceMsb; main [nm][n] over primes 0..nm-1."""
        a, ap = _ip(aux)
        main = np.ascontiguousarray(main, dtype=np.uint64)
        aux_poly = np.ascontiguousarray(aux_poly, dtype=np.uint64)
        nm = main.shape[0]
        out = np.empty_like(main)
        if mode == 0:
            lib().so_rns_scale_reduce(self._h, nm, ap, len(a), ctypes.c_uint64(t),
                                      int(main_ntt), _p(main), int(aux_ntt), _p(aux_poly),
                                      _p(out))
        elif mode == 1:
            lib().so_rns_approx_modreduce_lsb(self._h, nm, ap, len(a), ctypes.c_uint64(t),
                                              int(main_ntt), _p(main), int(aux_ntt),
                                              _p(aux_poly), _p(out))
        else:
            lib().so_rns_approx_modreduce_msb(self._h, nm, ap, len(a), int(main_ntt), _p(main),
                                              int(aux_ntt), _p(aux_poly), _p(out))
        return out

    def bfv_mul(self, nm, aux, t, a, b):
        """RnsBfvCiphertext::Mul: a, b [2][nm][n] -> [3][nm][n]."""
        x, xp = _ip(aux)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        out = np.empty((3, nm, self.n), np.uint64)
        lib().so_bfv_mul(self._h, nm, xp, len(x), ctypes.c_uint64(t), _p(a), _p(b), _p(out))
        return out

    def bfv_absorb(self, nm, aux, t, ct, pt):
        """RnsBfvCiphertext::AbsorbInPlace: ct [len][nm][n], pt [nm][n]."""
        x, xp = _ip(aux)
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        pt = np.ascontiguousarray(pt, dtype=np.uint64)
        out = np.empty_like(ct)
        lib().so_bfv_absorb(self._h, nm, xp, len(x), ctypes.c_uint64(t), ct.shape[0], _p(ct),
                            _p(pt), _p(out))
        return out

    def modreduce_lsb(self, poly, t, is_ntt=True):
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        L = poly.shape[0]
        out = np.empty((L - 1, self.n), np.uint64)
        st = lib().so_rns_modreduce_lsb(self._h, L, ctypes.c_uint64(int(t)), int(is_ntt),
                                        _p(poly), _p(out))
        if st:
            raise ValueError("ModReduceLsb cannot apply with only one prime modulus.")
        return out

    def mul_relin_batch(self, a, b, key_b, key_a, log_bs, threads=1):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        count, _, L, n = a.shape
        lb, p = _ip(log_bs)
        out = np.empty((count, 2, L, n), np.uint64)
        lib().so_rns_mul_relin_batch(self._h, L, p, _p(a), _p(b),
                                     _p(np.ascontiguousarray(key_b)),
                                     _p(np.ascontiguousarray(key_a)), _p(out), count, threads)
        return out


def compute_normalizer(k, log_t):
    return int(lib().so_compute_normalizer(k, log_t))


# ---------------------------------------------------------------------------
# Seeded input generation shared by tests, smoke and bench (splitmix64).
# ---------------------------------------------------------------------------
_M64 = (1 << 64) - 1


def splitmix64(seed, count):
    """count outputs of splitmix64 starting from state `seed` (vectorised)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed & _M64) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform_limbs(seed, qs, n, count=1):
    """Uniform residues mod each q (Montgomery reps are uniform too):
    shape [count][len(qs)][n]."""
    L = len(qs)
    raw = splitmix64(seed, count * L * n).reshape(count, L, n)
    q = np.array([int(x) for x in qs], dtype=np.uint64).reshape(1, L, 1)
    return raw % q


def prng_bytes(seed, start, count):
    """Bytes [start, start + count) of SHELL's ChaChaPrng stream of a 32-byte seed."""
    out = np.empty(count, np.uint8)
    lib().so_prng_bytes(bytes(seed), start, count, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return out


def chacha20_block(key, counter, nonce):
    """One RFC 7539 ChaCha20 keystream block."""
    out = np.empty(64, np.uint8)
    lib().so_chacha20_block(bytes(key), counter, bytes(nonce),
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return out.tobytes()
