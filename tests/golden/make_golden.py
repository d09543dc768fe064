#!/usr/bin/env python3
"""Generates tests/golden/*.npz and digests.json by running google/shell-encryption's
own code (oracle/_ref/libshellref.so, built from the reference sources in place by
oracle/ref/Makefile) on seeded inputs.

  make -C oracle/ref && python tests/golden/make_golden.py

Small cases are stored whole (inputs and outputs).  Full-size workloads are
stored as SHA-256 digests of the reference's outputs; their inputs are
regenerated from the recorded splitmix64 seeds (oracle.uniform_limbs).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402
from oracle import ref_oracle as R  # noqa: E402

Q45 = [35184371138561, 35184370941953, 35184370352129, 35184370155521,
       35184369893377, 35184368877569]
Q50 = [1125899904679937, 1125899903827969, 1125899903500289, 1125899903107073]
Q59 = 576460752303415297
Q60 = 1152921504606830593


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def main():
    if not R.available():
        sys.exit("oracle/_ref/libshellref.so is missing: run `make -C oracle/ref` first")
    g = {}
    # NTT tables and transforms (ntt_parameters.h, dft_transformations.h).
    for q, log_n in [(Q45[0], 1), (Q45[1], 4), (Q50[0], 7), (Q59, 12), (Q60, 12),
                     (Q45[2], 10), (Q45[0], 14)]:
        tag = f"ntt_{q}_{log_n}"
        f, i, ninv = R.prime_tables(q, log_n)
        x = O.uniform_limbs(1000 + log_n, [q], 1 << log_n, 2).reshape(2, -1)
        g[tag + "_psis_bitrev"] = f
        g[tag + "_psis_inv_bitrev"] = i
        g[tag + "_n_inv"] = np.array([ninv], np.uint64)
        g[tag + "_in"] = x
        g[tag + "_fwd"] = R.ntt(q, log_n, x)
        g[tag + "_inv"] = R.ntt(q, log_n, x, inverse=True)
    # RnsPolynomial::Substitute and ModReduceLsb.
    for log_n, qs, power in [(6, Q45[:3], 5), (10, Q50[:4], 1023)]:
        tag = f"subst_{log_n}_{power}"
        x = O.uniform_limbs(2000 + log_n, qs, 1 << log_n).reshape(len(qs), -1)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_in"] = x
        g[tag + "_out"] = R.rns_substitute(log_n, qs, x, power)
    for log_n, qs, is_ntt in [(5, Q45[:2], 1), (9, Q50[:4], 1), (9, Q50[:4], 0)]:
        tag = f"modreduce_{log_n}_{len(qs)}_{is_ntt}"
        x = O.uniform_limbs(3000 + log_n + is_ntt, qs, 1 << log_n).reshape(len(qs), -1)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_in"] = x
        g[tag + "_out"] = R.rns_modreduce_lsb(log_n, qs, x, 65537, bool(is_ntt))
    # BGV ct x ct + relinearization, and rotation (Substitute + Galois key).
    for log_n, qs, log_bs in [(5, Q45[:2], [20, 20]), (8, Q45[:3], [20, 20, 20]),
                              (7, Q50[:2], [50, 16])]:
        tag = f"mulrelin_{log_n}_{len(qs)}_{log_bs[-1]}"
        n = 1 << log_n
        k = O.Rns(log_n, qs).gadget_dim(log_bs)
        kb = O.uniform_limbs(4000 + log_n, qs, n, k)
        ka = O.uniform_limbs(4100 + log_n, qs, n, k)
        a = O.uniform_limbs(4200 + log_n, qs, n, 4).reshape(2, 2, len(qs), n)
        b = O.uniform_limbs(4300 + log_n, qs, n, 4).reshape(2, 2, len(qs), n)
        prod, out = R.bgv_mul_relin(log_n, qs, 65537, log_bs, kb, ka, a, b)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_log_bs"] = np.array(log_bs, np.int32)
        for nm, v in (("kb", kb), ("ka", ka), ("a", a), ("b", b), ("prod", prod), ("out", out)):
            g[f"{tag}_{nm}"] = v
        rtag = f"rotate_{log_n}_{len(qs)}_{log_bs[-1]}"
        power = 5
        g[rtag + "_power"] = np.array([power], np.int32)
        g[rtag + "_out"] = R.bgv_rotate(log_n, qs, log_bs, power, kb, ka, a)
    # RnsGaloisKey::PrecomputeRandomPad + ApplyToWithRandomPad.
    for log_n, qs, log_bs in [(6, Q45[:2], [20, 20]), (9, Q50[:3], [50, 16, 20])]:
        tag = f"galoispad_{log_n}_{len(qs)}"
        n, L = 1 << log_n, len(qs)
        k = O.Rns(log_n, qs).gadget_dim(log_bs)
        kb = O.uniform_limbs(6000 + log_n, qs, n, k)
        ka = O.uniform_limbs(6100 + log_n, qs, n, k)
        ct = O.uniform_limbs(6200 + log_n, qs, n, 4).reshape(2, 2, L, n)
        pad = O.uniform_limbs(6300 + log_n, qs, n, 2 * k).reshape(2, k, L, n)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_log_bs"] = np.array(log_bs, np.int32)
        for nm, v in (("kb", kb), ("ka", ka), ("ct", ct), ("pad", pad)):
            g[f"{tag}_{nm}"] = v
        g[tag + "_out"] = R.galois_random_pad(log_n, qs, log_bs, 5, kb, ka, ct, pad)
    # Oblivious expansion (n = 128, 60-bit q, base 2^10, 3 levels).
    q, log_n, levels, log_b = Q60, 7, 3, 10
    n = 1 << log_n
    dim = O.Prime(q, log_n).gadget_size(log_b)
    keys = O.uniform_limbs(5000, [q], n, levels * 2 * dim).reshape(levels, 2, dim, n)
    cts = O.uniform_limbs(5001, [q], n, 4).reshape(2, 2, n)
    g["expand_keys"] = keys
    g["expand_cts"] = cts
    g["expand_out"] = R.oblivious_expand(q, log_n, 16, levels, log_b, keys, cts)
    g["normalizer_10_16"] = np.array([R.compute_normalizer(10, 16)], np.uint64)
    # MontgomeryInt::SerializeVector bit streams (montgomery.cc:142-215),
    # including a 17- and a 31-bit modulus (streams that cross bytes oddly).
    for q, count in [(Q45[0], 1000), (Q50[3], 777), (Q59, 64), (Q60, 33), (65537, 101),
                     (2147483629, 57)]:
        v = O.splitmix64(8000 + count, count) % np.uint64(q)
        g[f"ser_{q}_values"] = v
        g[f"ser_{q}_bytes"] = R.serialize_vector(q, v)
    # SingleThreadChaChaPrng's stream (prng/chacha_prng_util.cc:30-98) across
    # two salt boundaries, and SampleUniform + SampleError drawn from it
    # (rns/rns_polynomial.h:638-667, rns/error_distribution.h:40-60); 65537
    # rejects about half of its 17-bit candidates.
    seed = bytes(range(40, 72))
    g["prng_seed"] = np.frombuffer(seed, np.uint8).copy()
    g["prng_bytes"] = R.prng_bytes(seed, 2 * 8160 + 100)
    for log_n, qs, var in [(6, [Q45[0], 65537], 1), (7, Q50[:2], 8), (5, [Q60], 256),
                           (6, Q45[:3], 33), (8, [65537], 3)]:
        tag = f"sample_{log_n}_{len(qs)}_{var}"
        sd = bytes((i * 7 + log_n + var) % 256 for i in range(32))
        a, e = R.sample_uniform_error(log_n, qs, var, sd)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_variance"] = np.array([var], np.int32)
        g[tag + "_seed"] = np.frombuffer(sd, np.uint8).copy()
        g[tag + "_a"] = a
        g[tag + "_e"] = e
    # RnsRlweSecretKey::EncryptPolynomialBgv (rns/rns_secret_key.h:188-231).
    for log_n, qs, t, var, count in [(6, Q45[:2], 65537, 8, 3), (10, [Q59], 2, 4, 2),
                                     (7, [Q45[0], 65537], 3, 1, 2)]:
        tag = f"encrypt_{log_n}_{len(qs)}"
        n, L = 1 << log_n, len(qs)
        key = O.uniform_limbs(9000 + log_n, qs, n).reshape(L, n)
        m = O.uniform_limbs(9100 + log_n, qs, n, count).reshape(count, L, n)
        seeds = [bytes((i * 13 + c * 5 + log_n) % 256 for i in range(32)) for c in range(count)]
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_params"] = np.array([t, var], np.uint64)
        g[tag + "_key"] = key
        g[tag + "_m"] = m
        g[tag + "_seeds"] = np.frombuffer(b"".join(seeds), np.uint8).reshape(count, 32).copy()
        g[tag + "_out"] = R.encrypt_bgv(log_n, qs, t, var, key, m, seeds)
    # Single-modulus symmetric RLWE (symmetric_encryption.h): SymmetricRlweKey::
    # Sample, Encrypt (each ciphertext with its own ChaCha PRNG; a and e are the
    # values Encrypt draws, replayed), ct + ct, ct * ct, absorb, Decrypt.
    for log_n, q, log_t, var, count in [(7, Q59, 16, 8, 4), (5, Q60, 2, 1, 2)]:
        tag = f"sym_{log_n}_{log_t}"
        n, t = 1 << log_n, (1 << log_t) + 1
        msgs = O.splitmix64(9900 + log_n, count * n).reshape(count, n) % np.uint64(t)
        key_seed = bytes((i * 11 + log_n) % 256 for i in range(32))
        seeds = [bytes((i * 17 + c * 3 + log_t) % 256 for i in range(32)) for c in range(count)]
        o = R.sym_c1(q, log_n, log_t, var, key_seed, seeds, msgs)
        g[tag + "_params"] = np.array([q, log_t, var], np.uint64)
        g[tag + "_msgs"] = msgs
        g[tag + "_key_seed"] = np.frombuffer(key_seed, np.uint8).copy()
        g[tag + "_seeds"] = np.frombuffer(b"".join(seeds), np.uint8).reshape(count, 32).copy()
        for nm, v in o.items():
            g[f"{tag}_{nm}"] = v
    # RnsGaloisKey::Compose (rns/rns_galois_key.cc:349-406).
    for log_n, qs, log_bs, p1, p2 in [(7, Q45[:2], [20, 20], 5, 25), (9, Q50[:3], [50, 16, 20],
                                                                       3, 7)]:
        tag = f"galcomp_{log_n}_{len(qs)}"
        n = 1 << log_n
        k = O.Rns(log_n, qs).gadget_dim(log_bs)
        keys = [O.uniform_limbs(6400 + log_n + 10 * i, qs, n, k) for i in range(4)]
        ob, oa, pw = R.galois_compose(log_n, qs, log_bs, p1, keys[0], keys[1], p2, keys[2],
                                      keys[3])
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_log_bs"] = np.array(log_bs, np.int32)
        g[tag + "_powers"] = np.array([p1, p2, pw], np.int32)
        for nm, v in zip(("kb1", "ka1", "kb2", "ka2"), keys):
            g[f"{tag}_{nm}"] = v
        g[tag + "_out_b"] = ob
        g[tag + "_out_a"] = oa
    # RNS basis conversion and BFV (rns/rns_polynomial.cc:349-852,
    # rns/rns_bfv_ciphertext.cc) on the reference's own BFV test parameters
    # (rns/testing/parameters.h GetBfvParametersForFiniteFieldEncoding).
    for tag, log_n, qs, ps, t in [("bfv_a", 11, [549755523073], [549755731969, 4169729], 40961),
                                  ("bfv_b", 11, [8589905921, 8589852673, 8589844481],
                                   [1073692673, 1073668097], 40961)]:
        n, L, K = 1 << log_n, len(qs), len(ps)
        x = O.uniform_limbs(9500 + L, qs, n).reshape(L, n)
        y = O.uniform_limbs(9600 + L, ps, n).reshape(K, n)
        g[tag + "_qs"] = np.array(qs, np.uint64)
        g[tag + "_ps"] = np.array(ps, np.uint64)
        g[tag + "_params"] = np.array([log_n, t], np.uint64)
        g[tag + "_x"] = x
        g[tag + "_y"] = y
        lv = L - 1
        g[tag + "_switch_up"] = R.switch_basis(log_n, qs, ps, lv, 0, x)
        g[tag + "_switch_down"] = R.switch_basis(log_n, qs, ps, lv, 1, y)
        g[tag + "_scale_up"] = R.switch_basis(log_n, qs, ps, lv, 2, x)
        g[tag + "_approx_down_ntt_bal"] = R.switch_basis(log_n, qs, ps, lv, 3, y, True, True)
        g[tag + "_approx_up"] = R.switch_basis(log_n, qs, ps, lv, 4, x, False, False)
        if L > 1:
            g[tag + "_modreduce_msb_ntt"] = R.modreduce_msb(log_n, qs, x, True)
            g[tag + "_modreduce_msb_coeff"] = R.modreduce_msb(log_n, qs, x, False)
        g[tag + "_scale_reduce"] = R.scale_reduce(log_n, qs, ps, t, 0, x, y, True, True)
        g[tag + "_approx_lsb"] = R.scale_reduce(log_n, qs, ps, t, 1, x, y, False, True)
        g[tag + "_approx_msb"] = R.scale_reduce(log_n, qs, ps, t, 2, x, y, True, False)
        a = O.uniform_limbs(9700 + L, qs, n, 4).reshape(2, 2, L, n)
        b = O.uniform_limbs(9800 + L, qs, n, 4).reshape(2, 2, L, n)
        g[tag + "_a"] = a
        g[tag + "_b"] = b
        g[tag + "_mul"] = R.bfv_mul(log_n, qs, ps, t, a, b)
        g[tag + "_absorb"] = R.bfv_absorb(log_n, qs, ps, t, a, x)
    np.savez_compressed(os.path.join(HERE, "reference_small.npz"), **g)

    # Full-size workloads: digests of the reference's outputs on seeded inputs.
    d = {}
    log_n, qs, log_bs = 14, Q45, [20] * 6
    n, k = 1 << log_n, 18
    kb = O.uniform_limbs(7001, qs, n, k)
    ka = O.uniform_limbs(7002, qs, n, k)
    a = O.uniform_limbs(7003, qs, n, 4).reshape(2, 2, 6, n)
    b = O.uniform_limbs(7004, qs, n, 4).reshape(2, 2, 6, n)
    prod, out = R.bgv_mul_relin(log_n, qs, 65537, log_bs, kb, ka, a, b)
    d["mul_relin_n14_L6"] = {
        "log_n": 14, "qs": qs, "t": 65537, "log_bs": log_bs, "count": 2,
        "seeds": {"key_b": 7001, "key_a": 7002, "a": 7003, "b": 7004},
        "prod_sha256": digest(prod), "out_sha256": digest(out)}
    rot = R.bgv_rotate(log_n, qs, log_bs, 5, kb, ka, a)
    d["rotate_n14_L6_p5"] = {"power": 5, "note": "key and ct as in mul_relin_n14_L6 (ct = a)",
                             "out_sha256": digest(rot)}
    x = O.uniform_limbs(7005, qs, n).reshape(6, n)
    d["modreduce_n14_L6"] = {"seed": 7005, "t": 65537,
                             "ntt_sha256": digest(R.rns_modreduce_lsb(log_n, qs, x, 65537, True)),
                             "coeff_sha256": digest(R.rns_modreduce_lsb(log_n, qs, x, 65537,
                                                                        False))}
    q, log_n, levels, log_b = Q60, 12, 10, 8
    n, dim = 1 << log_n, 8
    keys = O.uniform_limbs(7010, [q], n, levels * 2 * dim).reshape(levels, 2, dim, n)
    cts = O.uniform_limbs(7011, [q], n, 2).reshape(1, 2, n)
    d["expand_n12_levels10_b8"] = {"q": q, "log_n": 12, "levels": 10, "log_b": 8,
                                   "seeds": {"keys": 7010, "ct": 7011},
                                   "out_sha256": digest(R.oblivious_expand(q, log_n, 16, levels,
                                                                           log_b, keys, cts))}
    x = O.uniform_limbs(7020, [Q59], 1 << 12, 64).reshape(64, -1)
    d["ntt_q59_n12_x64"] = {"seed": 7020, "fwd_sha256": digest(R.ntt(Q59, 12, x)),
                            "inv_sha256": digest(R.ntt(Q59, 12, x, inverse=True))}
    log_n, qs, n = 14, Q45, 1 << 14
    key = O.uniform_limbs(7030, qs, n).reshape(6, n)
    m = O.uniform_limbs(7031, qs, n, 4).reshape(4, 6, n)
    seeds = [bytes([c + 1] * 32) for c in range(4)]
    d["encrypt_n14_L6"] = {"log_n": 14, "qs": qs, "t": 65537, "variance": 8, "count": 4,
                           "seeds": {"key": 7030, "m": 7031},
                           "prng_seeds": "ciphertext c: 32 bytes of value c + 1",
                           "out_sha256": digest(R.encrypt_bgv(log_n, qs, 65537, 8, key, m,
                                                              seeds))}
    P45 = [35184368320513, 35184368025601, 35184367828993, 35184367337473, 35184366911489,
           35184366551041, 35184366223361]
    a = O.uniform_limbs(7040, qs, n, 4).reshape(2, 2, 6, n)
    b = O.uniform_limbs(7041, qs, n, 4).reshape(2, 2, 6, n)
    d["bfv_mul_n14_L6_K7"] = {"log_n": 14, "qs": qs, "ps": P45, "t": 65537, "count": 2,
                              "seeds": {"a": 7040, "b": 7041},
                              "out_sha256": digest(R.bfv_mul(14, qs, P45, 65537, a, b))}
    # The symmetric flow at n = 2^12 with the 59-bit prime, t = 2^16 + 1,
    # 64 messages (the key's PRNG seed is 32 bytes of 200, ciphertext c's
    # 32 bytes of (7 c + 3) mod 256).
    log_n, count = 12, 64
    n = 1 << log_n
    msgs = O.splitmix64(7050, count * n).reshape(count, n) % np.uint64(65537)
    o = R.sym_c1(Q59, log_n, 16, 8, bytes([200] * 32),
                 [bytes([(7 * c + 3) % 256] * 32) for c in range(count)], msgs)
    ent = {"q": Q59, "log_n": log_n, "log_t": 16, "variance": 8, "count": count,
           "msgs": "splitmix64(7050) mod 65537, [count][n]",
           "prng_seeds": "key: 32 bytes of 200; ciphertext c: 32 bytes of (7c + 3) mod 256",
           "error": [float(x) for x in o["err"]]}
    for nm in ("s", "pt", "ct", "sum", "prod", "absorb", "dec", "dec_sum", "dec_prod",
               "dec_absorb"):
        ent[nm + "_sha256"] = digest(o[nm])
    d["sym_c1_n12_x64"] = ent
    # Error() bookkeeping of RNS ciphertexts (rns/rns_error_params.h and the
    # ciphertext / key-switch operations), two parameter sets.
    d["error_flow"] = []
    for log_n, qs, log_bs, log_t, sigma, e0, e1, scalar, power in [
            (10, Q45[:3], [20] * 3, 16, 3.19, 100.0, 250.0, 7, 5),
            (14, Q45, [20] * 6, 2, 1.5, 12.5, 3.25, 65537, 3)]:
        d["error_flow"].append({
            "log_n": log_n, "qs": qs, "log_bs": log_bs, "log_t": log_t, "sigma": sigma,
            "e0": e0, "e1": e1, "scalar": scalar, "power": power,
            "values": R.error_flow(log_n, qs, log_bs, log_t, sigma, e0, e1, scalar, power)})
    with open(os.path.join(HERE, "digests.json"), "w") as fh:
        json.dump(d, fh, indent=1)
    print("wrote", os.path.join(HERE, "reference_small.npz"), "and digests.json")


if __name__ == "__main__":
    main()
