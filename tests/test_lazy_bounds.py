"""Bounds behind the lazily reduced forward transforms, checked on the CPU.

The forward Cooley-Tukey butterflies of the device NTT (`bf_ct_lazy` in
csrc/ntt.cuh) skip every per-level reduction when all primes are below 2^58.
Their Shoup product (`shoup_lazy4` in csrc/modarith.cuh) forms the quotient
from three of the four 32x32 partial products of x * wp, so the remainder lies
in [0, 4q) instead of [0, 2q).  These tests restate that PTX sequence limb by
limb in Python and check it against exact integer arithmetic, and check the
growth bound (inputs below 2q, at most 4q per level, at most 15 levels: below
62 q < 2^64) and the key-switch chunk rule (chunk_lazy = floor(2^64 / (62 q_max))
products of a lazy digit and a key value stay below q * 2^64 for one REDC).
The other inline-PTX arithmetic (mulhi64, mac128, the exact fused shoup_lazy)
is restated the same way and checked against exact products.
"""
import random

import pytest

from conftest import P58, Q45, Q50, Q59, Q60

M32, M64 = (1 << 32) - 1, (1 << 64) - 1


def shoup_lazy4(x, w, wp, q):
    """The PTX of shoup_lazy4, one 32-bit instruction per line; returns
    (remainder mod 2^64, quotient estimate)."""
    nq = (-q) & M64
    xl, xh = x & M32, x >> 32
    wl, wh = w & M32, w >> 32
    pl, ph = wp & M32, wp >> 32
    nl, nh = nq & M32, nq >> 32
    h1 = (xh * pl) >> 32                    # mul.hi.u32 h1, xh, pl
    h2 = (xl * ph) >> 32                    # mul.hi.u32 h2, xl, ph
    s = h1 + h2                             # add.cc.u32 / addc.u32
    t = s                                   # mov.b64 t, {h1, h2}
    qq = (xh * ph + t) & M64                # mad.wide.u32 qq, xh, ph, t
    ql, qh = qq & M32, qq >> 32
    t = (xl * wl) & M64                     # mul.wide.u32 t, xl, wl
    t = (ql * nl + t) & M64                 # mad.wide.u32 t, ql, nl, t
    rl, rh = t & M32, t >> 32
    rh = (rh + xl * wh) & M32               # mad.lo.u32 rh, xl, wh, rh
    rh = (rh + xh * wl) & M32
    rh = (rh + ql * nh) & M32
    rh = (rh + qh * nl) & M32
    return (rh << 32) | rl, qq


PRIMES = [Q45[0], Q50[0], P58[0], Q59, Q60, 12289, (1 << 61) - 1]


@pytest.mark.parametrize("q", PRIMES)
def test_three_term_quotient(q):
    rng = random.Random(q)
    for _ in range(20000):
        w = rng.randrange(q)
        wp = (w << 64) // q
        x = rng.choice([rng.randrange(1 << 64), rng.randrange(62 * q) & M64, M64, 0, q - 1,
                        M64 - rng.randrange(1 << 40), rng.randrange(1 << 32) << 32])
        r, qe = shoup_lazy4(x, w, wp, q)
        exact = (x * wp) >> 64
        assert 0 <= exact - qe <= 2
        assert r == x * w - qe * q          # no wrap: the true remainder fits 64 bits
        assert r < 4 * q and r % q == x * w % q


def test_lazy_growth_fits_64_bits():
    # inputs below 2q, at most 4q added per level, n <= 2^15
    for q in P58 + [(1 << 58) - 1]:
        bound = 2 * q + 4 * q * 15
        assert bound == 62 * q and bound < 1 << 64
    # the encryption sink's REDC(x * t) and the digit inner product's REDC
    q = (1 << 58) - 1
    assert 62 * q * q < q << 64


@pytest.mark.parametrize("qs,k", [(Q45, 18), (P58[:2], 12), (Q50[:3], 9)])
def test_chunk_lazy_keeps_redc_input_below_q_2_64(qs, k):
    qmax = max(qs)
    chunk = max(1, min(k, M64 // (62 * qmax)))
    for q in qs:
        # chunk products of a lazy digit (< 62 q) and a key value (< q)
        assert chunk * (62 * q - 1) * (q - 1) < q << 64
    if qmax < 1 << 46:
        assert chunk == k                   # one REDC for all digits at 45-bit primes


def mulhi64(a, b):
    """csrc/modarith.cuh mulhi64: the four partial products on carry chains."""
    al, ah, bl, bh = a & M32, a >> 32, b & M32, b >> 32
    c1 = (al * bl) >> 32                                    # mul.hi.u32
    s = c1 + ((al * bh) & M32); c1, cy = s & M32, s >> 32   # mad.lo.cc
    c2 = (((al * bh) >> 32) + cy) & M32                     # madc.hi
    s = c1 + ((ah * bl) & M32); c1, cy = s & M32, s >> 32   # mad.lo.cc
    s = ((ah * bl) >> 32) + c2 + cy; c2, cy = s & M32, s >> 32  # madc.hi.cc
    c3 = cy                                                 # addc
    s = ((ah * bh) & M32) + c2; c2, cy = s & M32, s >> 32   # mad.lo.cc
    c3 = (((ah * bh) >> 32) + c3 + cy) & M32                # madc.hi
    return (c3 << 32) | c2


def mac128(lo, hi, a, b):
    """csrc/modarith.cuh mac128: (hi:lo) += a * b on three carry chains."""
    al, ah, bl, bh = a & M32, a >> 32, b & M32, b >> 32
    c = [lo & M32, lo >> 32, hi & M32, hi >> 32]
    s = c[0] + ((al * bl) & M32); c[0], cy = s & M32, s >> 32
    s = c[1] + ((al * bl) >> 32) + cy; c[1], cy = s & M32, s >> 32
    s = c[2] + ((ah * bh) & M32) + cy; c[2], cy = s & M32, s >> 32
    c[3] = (c[3] + ((ah * bh) >> 32) + cy) & M32
    for x, y in ((al, bh), (ah, bl)):
        s = c[1] + ((x * y) & M32); c[1], cy = s & M32, s >> 32
        s = c[2] + ((x * y) >> 32) + cy; c[2], cy = s & M32, s >> 32
        c[3] = (c[3] + cy) & M32
    return (c[1] << 32) | c[0], (c[3] << 32) | c[2]


def shoup_lazy(x, w, wp, q):
    """csrc/modarith.cuh shoup_lazy: exact quotient, fused x w + Q (2^64 - q)."""
    nq = (-q) & M64
    Q = mulhi64(x, wp)
    ql, qh = Q & M32, Q >> 32
    xl, xh, wl, wh, nl, nh = x & M32, x >> 32, w & M32, w >> 32, nq & M32, nq >> 32
    t = ((xl * wl) + ql * nl) & M64
    rl, rh = t & M32, t >> 32
    rh = (rh + xl * wh + xh * wl + ql * nh + qh * nl) & M32
    return (rh << 32) | rl


def test_carry_chain_products():
    rng = random.Random(7)
    for _ in range(20000):
        a = rng.choice([rng.randrange(1 << 64), M64, 0, rng.randrange(1 << 45)])
        b = rng.choice([rng.randrange(1 << 64), M64, 0, rng.randrange(1 << 45)])
        assert mulhi64(a, b) == (a * b) >> 64
        acc = rng.randrange(1 << 100)
        lo, hi = mac128(acc & M64, acc >> 64, a, b)
        assert (hi << 64) | lo == (acc + a * b) % (1 << 128)


@pytest.mark.parametrize("q", PRIMES)
def test_shoup_lazy_exact(q):
    rng = random.Random(q + 1)
    for _ in range(5000):
        w = rng.randrange(q)
        wp = (w << 64) // q
        x = rng.choice([rng.randrange(1 << 64), M64, 0, rng.randrange(4 * q) & M64])
        r = shoup_lazy(x, w, wp, q)
        assert r == x * w - ((x * wp) >> 64) * q and r < 2 * q


@pytest.mark.parametrize("q", [Q45[0], Q50[0], P58[0], (1 << 58) - 27])
def test_wide_inverse_butterfly_invariant(q):
    """bf_gs<WIDE> (csrc/ntt.cuh): inputs in [0, 4q) give outputs in [0, 4q)
    that agree mod q with the exact Gentleman-Sande butterfly."""
    assert 8 * q < 1 << 64
    rng = random.Random(q + 2)
    for _ in range(20000):
        w = rng.randrange(q)
        wp = (w << 64) // q
        X = rng.choice([rng.randrange(4 * q), 4 * q - 1, 0])
        Y = rng.choice([rng.randrange(4 * q), 4 * q - 1, 0])
        s = X + Y
        s = s - 4 * q if s >= 4 * q else s
        d = X - Y + 4 * q
        y, _ = shoup_lazy4(d, w, wp, q)
        assert 0 <= s < 4 * q and 0 <= y < 4 * q
        assert s % q == (X + Y) % q and y % q == (X - Y) * w % q
