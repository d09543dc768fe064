"""CPU tests of the oracle: the reference's own property tests re-expressed
against the C restatement (no GPU)."""
import numpy as np
import pytest

from conftest import Q45, Q50, Q59, Q60


def test_primes_are_the_configured_ones():
    sympy = pytest.importorskip("sympy")
    # 6 largest primes < 2^45 that are 1 mod 2^15
    got, x = [], (1 << 45) - ((1 << 45) % (1 << 15)) + 1
    while len(got) < 6:
        x -= 1 << 15
        if sympy.isprime(x):
            got.append(x)
    assert got == Q45
    got, x = [], (1 << 50) - ((1 << 50) % (1 << 16)) + 1
    while len(got) < 12:
        x -= 1 << 16
        if sympy.isprime(x):
            got.append(x)
    assert got == Q50
    assert sympy.isprime(Q59) and Q59 % (1 << 13) == 1 and Q59 < (1 << 59)
    assert sympy.isprime(Q60) and Q60 % (1 << 13) == 1 and Q60 < (1 << 60)


@pytest.mark.parametrize("q,log_n", [(Q59, 8), (Q45[0], 10), (Q60, 5)])
def test_ntt_roundtrip_and_tables(oracle, q, log_n):
    p = oracle.Prime(q, log_n)
    n = 1 << log_n
    x = oracle.uniform_limbs(3, [q], n).reshape(n)
    assert np.array_equal(p.ntt_inv(p.ntt_fwd(x)), x)
    info = p.info()
    psi = info["psi"]
    assert pow(psi, n, q) == q - 1
    fwd, inv = p.tables()
    plain_f = p.export(fwd)
    plain_i = p.export(inv)
    brv = [int(format(i, f"0{log_n}b")[::-1], 2) for i in range(n)]
    psi_inv = pow(psi, q - 2, q)
    for i in range(n):
        assert int(plain_f[i]) == pow(psi, brv[i], q)
        assert int(plain_i[i]) == pow(psi_inv, brv[i] + 1, q)


def test_ntt_delta(oracle):
    q, log_n = Q50[0], 9
    p = oracle.Prime(q, log_n)
    n = 1 << log_n
    x = np.zeros(n, np.uint64)
    x[0] = p.import_(np.array([1], np.uint64))[0]
    y = p.ntt_fwd(x)
    assert np.all(y == x[0])


def test_substitute_coefficient_domain(oracle):
    q, log_n, power = Q45[2], 5, 13
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    rng = np.random.default_rng(2)
    a = rng.integers(0, q, n, dtype=np.uint64)
    sub = p.export(p.ntt_inv(p.substitute(p.ntt_fwd(p.import_(a)), power)))
    want = [0] * n
    for i in range(n):
        e = (i * power) % (2 * n)
        if e >= n:
            want[e - n] = (want[e - n] - int(a[i])) % q
        else:
            want[e] = (want[e] + int(a[i])) % q
    assert [int(v) for v in sub] == want


def test_gadget_decompose_recomposes(oracle):
    """<g^{-1}(a), g> == a (rns/rns_gadget_test.cc)."""
    qs, log_n, log_bs = Q45[:3], 4, [20, 20, 20]
    rns = oracle.Rns(log_n, qs)
    n = 1 << log_n
    a = oracle.uniform_limbs(4, qs, n).reshape(3, n)
    digits = rns.decompose(a, log_bs)
    g = rns.gadget_vector(log_bs)
    acc = np.zeros_like(a)
    for j in range(digits.shape[0]):
        for l in range(3):
            acc[l] = rns.primes[l].fma(acc[l], digits[j, l],
                                        np.full(n, g[j, l], np.uint64))
    assert np.array_equal(acc, a)


def _bgv_setup(oracle, log_n, qs, t, seed):
    """Secret key, relin key (b_j = -a_j s + t e_j + g_j s^2) and helpers."""
    rng = np.random.default_rng(seed)
    n = 1 << log_n
    L = len(qs)
    rns = oracle.Rns(log_n, qs)

    def small(shape):  # centred binomial, variance 8 (sample_error.h:43-100)
        k = 16
        return (rng.integers(0, 2, shape + (k,)).sum(-1) -
                rng.integers(0, 2, shape + (k,)).sum(-1))

    def lift(vals):  # signed ints -> Montgomery limbs [L][n]
        out = np.empty((L, n), np.uint64)
        for l, q in enumerate(qs):
            out[l] = rns.primes[l].import_(np.array([int(v) % q for v in vals], np.uint64))
        return out

    s = rns.ntt_fwd(lift(small((n,))))
    return rns, s, small, lift, rng


def _enc(oracle, rns, s, small, lift, rng, m, t):
    qs, n = rns.qs, rns.n
    a = oracle.uniform_limbs(int(rng.integers(1 << 62)), qs, n).reshape(len(qs), n)
    e = rns.ntt_fwd(lift(small((n,))))
    mm = rns.ntt_fwd(lift(m))
    c0 = np.empty_like(a)
    c1 = np.empty_like(a)
    for l, p in enumerate(rns.primes):
        tt = p.import_(np.array([t], np.uint64))[0]
        c0[l] = p.fma(p.add(p.mul_scalar(e[l], tt), mm[l]), a[l], s[l])
        c1[l] = p.neg(a[l])
    return np.stack([c0, c1])


def _dec(rns, s, ct, t):
    acc = ct[0].copy()
    sp = s.copy()
    for i in range(1, ct.shape[0]):
        if i > 1:
            sp = np.stack([p.mul(sp[l], s[l]) for l, p in enumerate(rns.primes)])
        acc = np.stack([p.fma(acc[l], ct[i][l], sp[l]) for l, p in enumerate(rns.primes)])
    L = acc.shape[0]
    while L > 1:  # DecodeBgv: ModReduceLsb to q0 (coefficient_encoder.cc:74-108)
        acc = rns.modreduce_lsb(acc[:L], t, True)
        L -= 1
    q0 = rns.qs[0]
    v = rns.primes[0].export(rns.primes[0].ntt_inv(acc[0]))
    return np.array([((int(x) - q0) if int(x) > q0 // 2 else int(x)) % t for x in v])


def test_bgv_mul_relin_decrypts(oracle):
    """rns/rns_relinearization_key_test.cc: relin of a degree-2 product decrypts."""
    log_n, qs, t, log_bs = 5, Q45[:3], 65537, [20, 20, 20]
    rns, s, small, lift, rng = _bgv_setup(oracle, log_n, qs, t, 1)
    n = 1 << log_n
    k = rns.gadget_dim(log_bs)
    g = rns.gadget_vector(log_bs)
    s2 = np.stack([p.mul(s[l], s[l]) for l, p in enumerate(rns.primes)])
    ka = oracle.uniform_limbs(77, qs, n, k)
    kb = np.empty_like(ka)
    for j in range(k):
        e = rns.ntt_fwd(lift(small((n,))))
        for l, p in enumerate(rns.primes):
            tt = p.import_(np.array([t], np.uint64))[0]
            te = p.mul_scalar(e[l], tt)
            gs2 = p.mul_scalar(s2[l], g[j, l])
            kb[j, l] = p.sub(p.add(te, gs2), p.mul(ka[j, l], s[l]))
    m1 = rng.integers(0, t, n)
    m2 = rng.integers(0, t, n)
    c1 = _enc(oracle, rns, s, small, lift, rng, m1, t)
    c2 = _enc(oracle, rns, s, small, lift, rng, m2, t)
    prod = rns.tensor(c1, c2)
    out = rns.relin(prod, kb, ka, log_bs)
    want = np.zeros(n, dtype=object)
    for i in range(n):
        for j in range(n):
            v = int(m1[i]) * int(m2[j])
            if i + j >= n:
                want[i + j - n] -= v
            else:
                want[i + j] += v
    want = np.array([int(w) % t for w in want])
    assert np.array_equal(_dec(rns, s, out, t), want)
    assert np.array_equal(_dec(rns, s, prod, t), want)


def test_oblivious_expand_selects_index(oracle):
    """oblivious_expand_test.cc:219-259 at n=128, 60-bit q, log_t 16, base 2^10."""
    q, log_n, log_t, log_b, levels = Q60, 7, 16, 10, 3
    n = 1 << log_n
    t = (1 << log_t) + 1
    p = oracle.Prime(q, log_n)
    rng = np.random.default_rng(9)
    dim = p.gadget_size(log_b)

    def small():
        return rng.integers(0, 2, (n, 16)).sum(-1) - rng.integers(0, 2, (n, 16)).sum(-1)

    def imp(vals):
        return p.import_(np.array([int(v) % q for v in vals], np.uint64))

    s = p.ntt_fwd(imp(small()))
    tt = p.import_(np.array([t], np.uint64))[0]

    def enc(m_ntt, key):
        a = oracle.uniform_limbs(int(rng.integers(1 << 62)), [q], n).reshape(n)
        e = p.ntt_fwd(imp(small()))
        c0 = p.fma(p.add(p.mul_scalar(e, tt), m_ntt), a, key)
        return np.stack([c0, p.neg(a)])

    keys = np.empty((levels, 2, dim, n), np.uint64)
    for j in range(levels):
        power = (n >> j) + 1
        s_sub = p.substitute(s, power)  # key for s(X^power) -> s
        for d in range(dim):
            r = oracle.uniform_limbs(int(rng.integers(1 << 62)), [q], n).reshape(n)
            e = p.ntt_fwd(imp(small()))
            bd = p.mul_scalar(s_sub, p.import_(np.array([pow(2, log_b * d, q)], np.uint64))[0])
            keys[j, 0, d] = p.add(p.add(p.mul_scalar(e, tt), p.neg(p.mul(r, s))), bd)
            keys[j, 1, d] = r
    idx = 5
    mono = np.zeros(n, dtype=object)
    mono[idx] = oracle.compute_normalizer(levels, log_t)
    ct = enc(p.ntt_fwd(imp(mono)), s)
    out = p.oblivious_expand(levels, log_b, keys, ct)
    for i in range(1 << levels):
        v = p.export(p.ntt_inv(p.fma(out[i, 0], out[i, 1], s)))
        dec = [((int(x) - q) if int(x) > q // 2 else int(x)) % t for x in v]
        assert dec[0] == (1 if i == idx else 0)
        assert all(d == 0 for d in dec[1:])


def test_symmetric_encrypt_decrypt_round_trip(oracle):
    """decrypt(encrypt(m)) == m and decrypt(ct1 + ct2) == m1 + m2 mod t
    (symmetric_encryption_test.cc's round-trip and additive properties)."""
    q, log_n, t = 576460752303415297, 10, 65537
    n = 1 << log_n
    p = oracle.Prime(q, log_n)
    rng = np.random.default_rng(5)

    def cbd():
        b = rng.integers(0, 2, size=(n, 32))
        return b[:, :16].sum(1) - b[:, 16:].sum(1)

    def mont(v):
        return p.import_(np.array([int(x) % q for x in v], dtype=np.uint64))

    s = p.ntt_fwd(mont(cbd()))
    m1, m2 = rng.integers(0, t, n), rng.integers(0, t, n)
    c1 = p.sym_encrypt(t, s, oracle.uniform_limbs(1, [q], n, 1).reshape(n), mont(cbd()),
                       p.ntt_fwd(mont(m1)))
    c2 = p.sym_encrypt(t, s, oracle.uniform_limbs(2, [q], n, 1).reshape(n), mont(cbd()),
                       p.ntt_fwd(mont(m2)))
    assert np.array_equal(p.sym_decrypt(t, s, c1).astype(np.int64), m1)
    assert np.array_equal(p.sym_decrypt(t, s, p.add(c1, c2)).astype(np.int64), (m1 + m2) % t)


def test_chacha20_block_rfc7539(oracle):
    """RFC 7539 section 2.3.2's test vector for the block function."""
    key = bytes(range(32))
    nonce = bytes.fromhex("000000090000004a00000000")
    want = bytes.fromhex("10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
                         "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")
    assert oracle.chacha20_block(key, 1, nonce) == want


def test_chacha_prng_stream_matches_cryptography(oracle):
    """The PRNG stream (prng/chacha_prng_util.cc:30-98): salt s gives 8160
    bytes of ChaCha20 keystream under nonce "salt" || LE64(s), counter 0 --
    checked against an independent ChaCha20 (Python `cryptography`)."""
    ciphers = pytest.importorskip("cryptography.hazmat.primitives.ciphers")
    seed = bytes(range(100, 132))
    got = oracle.prng_bytes(seed, 0, 3 * 8160 + 77).tobytes()
    want = b""
    for salt in range(4):
        nonce = (0).to_bytes(4, "little") + b"salt" + salt.to_bytes(8, "little")
        enc = ciphers.Cipher(ciphers.algorithms.ChaCha20(seed, nonce), mode=None).encryptor()
        want += enc.update(bytes(8160))
    assert got == want[: len(got)]
    # an unaligned window
    assert oracle.prng_bytes(seed, 8155, 20).tobytes() == want[8155:8175]


@pytest.mark.parametrize("variance", [1, 3, 4, 8, 33, 256])
def test_sample_error_distribution(oracle, variance):
    """SampleError's centred binomial: |e| <= 2 * variance, mean ~0 and
    variance ~`variance` (sample_error.h:43-100)."""
    q, log_n = Q45[0], 12
    n = 1 << log_n
    r = oracle.Rns(log_n, [q])
    p = oracle.Prime(q, log_n)
    _, e = r.sample_uniform_error(1, variance, bytes([variance % 256] * 32))
    v = p.export(p.ntt_inv(e[0])).astype(object)
    s = np.array([int(x) - q if int(x) > q // 2 else int(x) for x in v], dtype=np.int64)
    assert np.abs(s).max() <= 2 * variance
    assert abs(s.mean()) < 6 * np.sqrt(variance / n)
    assert abs(s.var() / variance - 1) < 0.15


def test_sample_uniform_in_range(oracle):
    """SampleUniform: every value below its prime, 65537 (half the 17-bit
    candidates rejected) included."""
    qs = [Q45[0], 65537]
    r = oracle.Rns(10, qs)
    a, _ = r.sample_uniform_error(2, 8, bytes(32))
    for l, q in enumerate(qs):
        assert int(a[l].max()) < q
        assert len(np.unique(a[l])) > (1 << 10) * 0.9 if q > 1 << 20 else True
