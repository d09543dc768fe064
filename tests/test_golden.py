"""Golden vectors produced by google/shell-encryption's own code (compiled in
place by oracle/ref/Makefile; generator: tests/golden/make_golden.py).

CPU tests pin the C restatement (oracle/shell_oracle.c) to the reference;
the gpu-marked tests check the CUDA library against the same vectors
through the C ABI.  Full-size workloads are compared as SHA-256 digests of
outputs on seeded inputs.
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")
SMALL = np.load(os.path.join(GOLDEN, "reference_small.npz"))
DIGESTS = json.load(open(os.path.join(GOLDEN, "digests.json")))


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def tags(prefix):
    return sorted({k.rsplit("_", 1)[0] for k in SMALL.files if k.startswith(prefix) and
                   k.endswith("_in")})


NTT_TAGS = sorted({k[:-3] for k in SMALL.files if k.startswith("ntt_") and k.endswith("_in")})


def _ntt_params(tag):
    _, q, log_n = tag.split("_")
    return int(q), int(log_n)


# --------------------------------------------------------------------------
# The oracle restatement against the reference (CPU)
# --------------------------------------------------------------------------

@pytest.mark.parametrize("tag", NTT_TAGS)
def test_oracle_ntt_golden(oracle, tag):
    q, log_n = _ntt_params(tag)
    p = oracle.Prime(q, log_n)
    f, i = p.tables()
    assert np.array_equal(f, SMALL[tag + "_psis_bitrev"])
    assert np.array_equal(i, SMALL[tag + "_psis_inv_bitrev"])
    assert p.info()["n_inv"] == int(SMALL[tag + "_n_inv"][0])
    x = SMALL[tag + "_in"]
    assert np.array_equal(np.stack([p.ntt_fwd(r) for r in x]), SMALL[tag + "_fwd"])
    assert np.array_equal(np.stack([p.ntt_inv(r) for r in x]), SMALL[tag + "_inv"])


def _cases(prefix):
    return sorted({k[:k.index("_qs")] for k in SMALL.files if k.startswith(prefix) and
                   k.endswith("_qs")})


@pytest.mark.parametrize("tag", _cases("subst_"))
def test_oracle_substitute_golden(oracle, tag):
    log_n, power = int(tag.split("_")[1]), int(tag.split("_")[2])
    rns = oracle.Rns(log_n, SMALL[tag + "_qs"])
    assert np.array_equal(rns.substitute(SMALL[tag + "_in"], power), SMALL[tag + "_out"])


@pytest.mark.parametrize("tag", _cases("modreduce_"))
def test_oracle_modreduce_golden(oracle, tag):
    log_n, is_ntt = int(tag.split("_")[1]), int(tag.split("_")[3])
    rns = oracle.Rns(log_n, SMALL[tag + "_qs"])
    got = rns.modreduce_lsb(SMALL[tag + "_in"], 65537, bool(is_ntt))
    assert np.array_equal(got, SMALL[tag + "_out"])


@pytest.mark.parametrize("tag", _cases("mulrelin_"))
def test_oracle_mul_relin_and_rotate_golden(oracle, tag):
    log_n = int(tag.split("_")[1])
    qs = SMALL[tag + "_qs"]
    lb = SMALL[tag + "_log_bs"]
    rns = oracle.Rns(log_n, qs)
    a, b, kb, ka = (SMALL[f"{tag}_{x}"] for x in ("a", "b", "kb", "ka"))
    prod = np.stack([rns.tensor(a[i], b[i]) for i in range(a.shape[0])])
    assert np.array_equal(prod, SMALL[tag + "_prod"])
    assert np.array_equal(rns.mul_relin_batch(a, b, kb, ka, lb), SMALL[tag + "_out"])
    rtag = tag.replace("mulrelin_", "rotate_")
    power = int(SMALL[rtag + "_power"][0])
    sub = np.stack([np.stack([rns.substitute(a[i, c], power) for c in range(2)])
                    for i in range(a.shape[0])])
    rot = np.stack([rns.galois(sub[i], kb, ka, lb) for i in range(a.shape[0])])
    assert np.array_equal(rot, SMALL[rtag + "_out"])


def test_oracle_expand_golden(oracle):
    from conftest import Q60
    p = oracle.Prime(Q60, 7)
    keys, cts = SMALL["expand_keys"], SMALL["expand_cts"]
    got = np.stack([p.oblivious_expand(3, 10, keys, cts[i]) for i in range(cts.shape[0])])
    assert np.array_equal(got, SMALL["expand_out"])
    assert oracle.compute_normalizer(10, 16) == int(SMALL["normalizer_10_16"][0])


def test_oracle_full_size_digests(oracle):
    d = DIGESTS["mul_relin_n14_L6"]
    qs, n = d["qs"], 1 << d["log_n"]
    rns = oracle.Rns(d["log_n"], qs)
    s = d["seeds"]
    kb = oracle.uniform_limbs(s["key_b"], qs, n, 18)
    ka = oracle.uniform_limbs(s["key_a"], qs, n, 18)
    a = oracle.uniform_limbs(s["a"], qs, n, 4).reshape(2, 2, 6, n)
    b = oracle.uniform_limbs(s["b"], qs, n, 4).reshape(2, 2, 6, n)
    prod = np.stack([rns.tensor(a[i], b[i]) for i in range(2)])
    assert digest(prod) == d["prod_sha256"]
    assert digest(rns.mul_relin_batch(a, b, kb, ka, d["log_bs"], threads=2)) == d["out_sha256"]
    sub = np.stack([np.stack([rns.substitute(a[i, c], 5) for c in range(2)]) for i in range(2)])
    rot = np.stack([rns.galois(sub[i], kb, ka, d["log_bs"]) for i in range(2)])
    assert digest(rot) == DIGESTS["rotate_n14_L6_p5"]["out_sha256"]
    m = DIGESTS["modreduce_n14_L6"]
    x = oracle.uniform_limbs(m["seed"], qs, n).reshape(6, n)
    assert digest(rns.modreduce_lsb(x, 65537, True)) == m["ntt_sha256"]
    assert digest(rns.modreduce_lsb(x, 65537, False)) == m["coeff_sha256"]


def test_oracle_expand_full_size_digest(oracle):
    d = DIGESTS["expand_n12_levels10_b8"]
    n = 1 << d["log_n"]
    p = oracle.Prime(d["q"], d["log_n"])
    keys = oracle.uniform_limbs(d["seeds"]["keys"], [d["q"]], n, d["levels"] * 2 * 8).reshape(
        d["levels"], 2, 8, n)
    ct = oracle.uniform_limbs(d["seeds"]["ct"], [d["q"]], n, 2).reshape(2, n)
    out = p.oblivious_expand(d["levels"], d["log_b"], keys, ct)
    assert digest(out[None]) == d["out_sha256"]


def test_oracle_matches_reference_library_when_built(oracle):
    """Where the reference sources are present (this build container), also
    compare directly with the shim-built reference on fresh inputs."""
    from oracle import ref_oracle as R
    if not R.available():
        pytest.skip("oracle/_ref not built (reference sources absent)")
    from conftest import Q45
    qs, log_n, log_bs = Q45[:4], 9, [20] * 4
    rns = oracle.Rns(log_n, qs)
    n = 1 << log_n
    k = rns.gadget_dim(log_bs)
    kb, ka = oracle.uniform_limbs(31, qs, n, k), oracle.uniform_limbs(32, qs, n, k)
    a = oracle.uniform_limbs(33, qs, n, 6).reshape(3, 2, 4, n)
    b = oracle.uniform_limbs(34, qs, n, 6).reshape(3, 2, 4, n)
    _, ref_out = R.bgv_mul_relin(log_n, qs, 65537, log_bs, kb, ka, a, b)
    assert np.array_equal(rns.mul_relin_batch(a, b, kb, ka, log_bs), ref_out)


# --------------------------------------------------------------------------
# The CUDA library against the reference's vectors (GPU)
# --------------------------------------------------------------------------

def _run(sg, fn, *args):
    sg.check(fn(*args))
    sg.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", NTT_TAGS)
def test_gpu_ntt_golden(sg, tag):
    q, log_n = _ntt_params(tag)
    ctx = sg.Context(log_n, [q])
    f, i = ctx.ntt_tables(0)
    assert np.array_equal(f, SMALL[tag + "_psis_bitrev"])
    assert np.array_equal(i, SMALL[tag + "_psis_inv_bitrev"])
    x = SMALL[tag + "_in"]
    d = sg.DeviceBuffer.from_array(x)
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, d.ptr, x.shape[0], 1, None)
    assert np.array_equal(d.download(x.shape), SMALL[tag + "_fwd"])
    d.upload(x)
    _run(sg, sg.lib().shg_ntt_inverse, ctx.h, d.ptr, x.shape[0], 1, None)
    assert np.array_equal(d.download(x.shape), SMALL[tag + "_inv"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag", _cases("subst_"))
def test_gpu_substitute_golden(sg, tag):
    log_n, power = int(tag.split("_")[1]), int(tag.split("_")[2])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    ctx = sg.Context(log_n, qs)
    x = SMALL[tag + "_in"]
    d, out = sg.DeviceBuffer.from_array(x), sg.DeviceBuffer(x.nbytes)
    _run(sg, sg.lib().shg_poly_substitute, ctx.h, out.ptr, d.ptr, power, 1, len(qs), None)
    assert np.array_equal(out.download(x.shape), SMALL[tag + "_out"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag", _cases("modreduce_"))
def test_gpu_modreduce_golden(sg, tag):
    log_n, is_ntt = int(tag.split("_")[1]), int(tag.split("_")[3])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    ctx = sg.Context(log_n, qs, 65537)
    ql_inv = ctx.ql_inv(len(qs) - 1)
    x = SMALL[tag + "_in"]
    want = SMALL[tag + "_out"]
    d, out = sg.DeviceBuffer.from_array(x), sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_poly_modreduce_lsb, ctx.h, out.ptr, d.ptr, 65537,
         ql_inv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), is_ntt, 1, len(qs), None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", _cases("mulrelin_"))
def test_gpu_mul_relin_and_rotate_golden(sg, tag):
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    lb = [int(x) for x in SMALL[tag + "_log_bs"]]
    a, b, kb, ka = (SMALL[f"{tag}_{x}"] for x in ("a", "b", "kb", "ka"))
    count = a.shape[0]
    ctx = sg.Context(log_n, qs)
    key = sg.Key(ctx, lb, 1, kb, ka)
    lib = sg.lib()
    da, db = sg.DeviceBuffer.from_array(a), sg.DeviceBuffer.from_array(b)
    prod = sg.DeviceBuffer(SMALL[tag + "_prod"].nbytes)
    out = sg.DeviceBuffer(a.nbytes)
    _run(sg, lib.shg_ct_tensor, ctx.h, prod.ptr, da.ptr, db.ptr, count, len(qs), None)
    assert np.array_equal(prod.download(SMALL[tag + "_prod"].shape), SMALL[tag + "_prod"])
    _run(sg, lib.shg_relin_apply, ctx.h, key.h, out.ptr, prod.ptr, count, None)
    assert np.array_equal(out.download(a.shape), SMALL[tag + "_out"])
    _run(sg, lib.shg_bgv_mul_relin, ctx.h, key.h, out.ptr, da.ptr, db.ptr, count, None)
    assert np.array_equal(out.download(a.shape), SMALL[tag + "_out"])
    rtag = tag.replace("mulrelin_", "rotate_")
    power = int(SMALL[rtag + "_power"][0])
    gkey = sg.Key(ctx, lb, power, kb, ka)
    _run(sg, lib.shg_bgv_rotate, ctx.h, gkey.h, out.ptr, da.ptr, count, None)
    assert np.array_equal(out.download(a.shape), SMALL[rtag + "_out"])


@pytest.mark.gpu
def test_gpu_expand_golden(sg):
    from conftest import Q60
    keys, cts, want = SMALL["expand_keys"], SMALL["expand_cts"], SMALL["expand_out"]
    ctx = sg.Context(7, [Q60])
    gk = [sg.Key(ctx, [10], (128 >> j) + 1, keys[j, 0], keys[j, 1]) for j in range(3)]
    arr = (ctypes.c_void_p * 3)(*[k.h for k in gk])
    d, out = sg.DeviceBuffer.from_array(cts), sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_oblivious_expand, ctx.h, arr, 3, out.ptr, d.ptr, cts.shape[0], None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.gpu
def test_gpu_full_size_digests(sg, oracle):
    d = DIGESTS["mul_relin_n14_L6"]
    qs, n = d["qs"], 1 << d["log_n"]
    s = d["seeds"]
    kb = oracle.uniform_limbs(s["key_b"], qs, n, 18)
    ka = oracle.uniform_limbs(s["key_a"], qs, n, 18)
    a = oracle.uniform_limbs(s["a"], qs, n, 4).reshape(2, 2, 6, n)
    b = oracle.uniform_limbs(s["b"], qs, n, 4).reshape(2, 2, 6, n)
    ctx = sg.Context(d["log_n"], qs, d["t"])
    key = sg.Key(ctx, d["log_bs"], 1, kb, ka)
    lib = sg.lib()
    da, db = sg.DeviceBuffer.from_array(a), sg.DeviceBuffer.from_array(b)
    out = sg.DeviceBuffer(a.nbytes)
    prod = sg.DeviceBuffer(3 * 6 * n * 8 * 2)
    _run(sg, lib.shg_ct_tensor, ctx.h, prod.ptr, da.ptr, db.ptr, 2, 6, None)
    assert digest(prod.download((2, 3, 6, n))) == d["prod_sha256"]
    _run(sg, lib.shg_bgv_mul_relin, ctx.h, key.h, out.ptr, da.ptr, db.ptr, 2, None)
    assert digest(out.download(a.shape)) == d["out_sha256"]
    gkey = sg.Key(ctx, d["log_bs"], 5, kb, ka)
    _run(sg, lib.shg_bgv_rotate, ctx.h, gkey.h, out.ptr, da.ptr, 2, None)
    assert digest(out.download(a.shape)) == DIGESTS["rotate_n14_L6_p5"]["out_sha256"]
    m = DIGESTS["modreduce_n14_L6"]
    x = oracle.uniform_limbs(m["seed"], qs, n).reshape(1, 6, n)
    dx, dout = sg.DeviceBuffer.from_array(x), sg.DeviceBuffer(5 * n * 8)
    ql_inv = ctx.ql_inv(5)
    for is_ntt, key_name in ((1, "ntt_sha256"), (0, "coeff_sha256")):
        _run(sg, lib.shg_poly_modreduce_lsb, ctx.h, dout.ptr, dx.ptr, 65537,
             ql_inv.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), is_ntt, 1, 6, None)
        assert digest(dout.download((5, n))) == m[key_name]


@pytest.mark.gpu
def test_gpu_expand_full_size_digest(sg, oracle):
    d = DIGESTS["expand_n12_levels10_b8"]
    q, log_n, levels = d["q"], d["log_n"], d["levels"]
    n = 1 << log_n
    keys = oracle.uniform_limbs(d["seeds"]["keys"], [q], n, levels * 2 * 8).reshape(
        levels, 2, 8, n)
    ct = oracle.uniform_limbs(d["seeds"]["ct"], [q], n, 2).reshape(1, 2, n)
    ctx = sg.Context(log_n, [q])
    gk = [sg.Key(ctx, [d["log_b"]], (n >> j) + 1, keys[j, 0], keys[j, 1])
          for j in range(levels)]
    arr = (ctypes.c_void_p * levels)(*[k.h for k in gk])
    dct = sg.DeviceBuffer.from_array(ct)
    out = sg.DeviceBuffer(2 * n * 8 << levels)
    _run(sg, sg.lib().shg_oblivious_expand, ctx.h, arr, levels, out.ptr, dct.ptr, 1, None)
    assert digest(out.download((1, 1 << levels, 2, n))) == d["out_sha256"]


@pytest.mark.gpu
def test_gpu_ntt_q59_digest(sg, oracle):
    from conftest import Q59
    d = DIGESTS["ntt_q59_n12_x64"]
    x = oracle.uniform_limbs(d["seed"], [Q59], 1 << 12, 64).reshape(64, 1, -1)
    ctx = sg.Context(12, [Q59])
    buf = sg.DeviceBuffer.from_array(x)
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, buf.ptr, 64, 1, None)
    assert digest(buf.download((64, 1 << 12))) == d["fwd_sha256"]
    buf.upload(x)
    _run(sg, sg.lib().shg_ntt_inverse, ctx.h, buf.ptr, 64, 1, None)
    assert digest(buf.download((64, 1 << 12))) == d["inv_sha256"]


SER_TAGS = sorted({k[len("ser_"):-len("_values")] for k in SMALL.files
                   if k.startswith("ser_") and k.endswith("_values")})


@pytest.mark.parametrize("q", SER_TAGS)
def test_oracle_serialization_golden(oracle, q):
    """MontgomeryInt::SerializeVector / DeserializeVector streams of the
    reference (17- to 60-bit moduli)."""
    v = SMALL[f"ser_{q}_values"]
    want = SMALL[f"ser_{q}_bytes"]
    p = oracle.Prime(int(q), 1)
    assert np.array_equal(p.serialize(v), want)
    assert np.array_equal(p.deserialize(want, v.size), v)


PAD_TAGS = sorted({k[:-len("_out")] for k in SMALL.files
                   if k.startswith("galoispad_") and k.endswith("_out")})


@pytest.mark.parametrize("tag", PAD_TAGS)
def test_oracle_galois_random_pad_golden(oracle, tag):
    """RnsGaloisKey::PrecomputeRandomPad + ApplyToWithRandomPad of the reference."""
    _, log_n, _ = tag.split("_")
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    rns = oracle.Rns(int(log_n), qs)
    ct, pad = SMALL[tag + "_ct"], SMALL[tag + "_pad"]
    got = np.stack([rns.galois_pad(ct[i], pad[i], SMALL[tag + "_kb"], SMALL[tag + "_ka"])
                    for i in range(ct.shape[0])])
    assert np.array_equal(got, SMALL[tag + "_out"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag", PAD_TAGS)
def test_gpu_galois_random_pad_golden(sg, tag):
    """Device PrecomputeRandomPad + ApplyToWithRandomPad against the reference."""
    _, log_n, _ = tag.split("_")
    log_n = int(log_n)
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    lib = sg.lib()
    ctx = sg.Context(log_n, qs)
    key = sg.Key(ctx, [int(b) for b in SMALL[tag + "_log_bs"]], 5, SMALL[tag + "_kb"],
                 SMALL[tag + "_ka"])
    ct, pad, want = SMALL[tag + "_ct"], SMALL[tag + "_pad"], SMALL[tag + "_out"]
    count, L, n = ct.shape[0], ct.shape[2], ct.shape[3]
    dct, dpad = sg.DeviceBuffer.from_array(ct), sg.DeviceBuffer.from_array(pad)
    dnew = sg.DeviceBuffer(count * L * n * 8)
    sg.check(lib.shg_galois_precompute_pad(ctx.h, key.h, dnew.ptr, dpad.ptr, count, None))
    out = sg.DeviceBuffer(want.nbytes)
    sg.check(lib.shg_galois_apply_with_pad(ctx.h, key.h, out.ptr, dct.ptr, dpad.ptr, dnew.ptr,
                                           count, None))
    sg.synchronize()
    assert np.array_equal(out.download(want.shape), want)


# --------------------------------------------------------------------------
# ChaCha PRNG, SampleUniform / SampleError and EncryptPolynomialBgv
# --------------------------------------------------------------------------

SAMPLE_TAGS = sorted({k[:-len("_a")] for k in SMALL.files
                      if k.startswith("sample_") and k.endswith("_a")})
ENC_TAGS = sorted({k[:-len("_out")] for k in SMALL.files
                   if k.startswith("encrypt_") and k.endswith("_out")})


def _seed_words(seeds):
    """32-byte seeds as the uint64 words a device buffer holds (byte order kept)."""
    return np.frombuffer(np.ascontiguousarray(seeds, dtype=np.uint8).tobytes(), np.uint64)


def test_oracle_prng_golden(oracle):
    """SingleThreadChaChaPrng's byte stream across two salt boundaries."""
    seed = SMALL["prng_seed"].tobytes()
    want = SMALL["prng_bytes"]
    assert np.array_equal(oracle.prng_bytes(seed, 0, want.size), want)
    assert np.array_equal(oracle.prng_bytes(seed, 8150, 30), want[8150:8180])


@pytest.mark.parametrize("tag", SAMPLE_TAGS)
def test_oracle_sample_uniform_error_golden(oracle, tag):
    """RnsPolynomial::SampleUniform then SampleError of the reference."""
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    a, e = oracle.Rns(log_n, qs).sample_uniform_error(
        len(qs), int(SMALL[tag + "_variance"][0]), SMALL[tag + "_seed"].tobytes())
    assert np.array_equal(a, SMALL[tag + "_a"])
    assert np.array_equal(e, SMALL[tag + "_e"])


@pytest.mark.parametrize("tag", ENC_TAGS)
def test_oracle_encrypt_bgv_golden(oracle, tag):
    """RnsRlweSecretKey::EncryptPolynomialBgv of the reference."""
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    t, var = (int(x) for x in SMALL[tag + "_params"])
    rns = oracle.Rns(log_n, qs)
    m, seeds = SMALL[tag + "_m"], SMALL[tag + "_seeds"]
    got = np.stack([rns.encrypt_bgv(t, var, SMALL[tag + "_key"], m[i], seeds[i].tobytes())
                    for i in range(m.shape[0])])
    assert np.array_equal(got, SMALL[tag + "_out"])


def _encrypt_digest_inputs(oracle):
    d = DIGESTS["encrypt_n14_L6"]
    n, qs = 1 << d["log_n"], d["qs"]
    key = oracle.uniform_limbs(d["seeds"]["key"], qs, n).reshape(6, n)
    m = oracle.uniform_limbs(d["seeds"]["m"], qs, n, d["count"]).reshape(d["count"], 6, n)
    seeds = np.array([[c + 1] * 32 for c in range(d["count"])], np.uint8)
    return d, key, m, seeds


def test_oracle_encrypt_full_size_digest(oracle):
    d, key, m, seeds = _encrypt_digest_inputs(oracle)
    rns = oracle.Rns(d["log_n"], d["qs"])
    got = np.stack([rns.encrypt_bgv(d["t"], d["variance"], key, m[i], seeds[i].tobytes())
                    for i in range(d["count"])])
    assert digest(got) == d["out_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("tag", SAMPLE_TAGS)
def test_gpu_sample_uniform_error_golden(sg, tag):
    """Device SampleUniform + SampleError against the reference."""
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    want_a, want_e = SMALL[tag + "_a"], SMALL[tag + "_e"]
    ctx = sg.Context(log_n, qs)
    da, de = sg.DeviceBuffer(want_a.nbytes), sg.DeviceBuffer(want_e.nbytes)
    ds = sg.DeviceBuffer.from_array(_seed_words(SMALL[tag + "_seed"]))
    _run(sg, sg.lib().shg_sample_uniform_error, ctx.h, da.ptr, de.ptr, ds.ptr, len(qs), 1,
         int(SMALL[tag + "_variance"][0]), None)
    assert np.array_equal(da.download(want_a.shape), want_a)
    assert np.array_equal(de.download(want_e.shape), want_e)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ENC_TAGS)
def test_gpu_encrypt_bgv_golden(sg, tag):
    """Device EncryptPolynomialBgv against the reference."""
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    t, var = (int(x) for x in SMALL[tag + "_params"])
    want, m = SMALL[tag + "_out"], SMALL[tag + "_m"]
    ctx = sg.Context(log_n, qs, t)
    dk, dm = sg.DeviceBuffer.from_array(SMALL[tag + "_key"]), sg.DeviceBuffer.from_array(m)
    ds = sg.DeviceBuffer.from_array(_seed_words(SMALL[tag + "_seeds"]))
    out = sg.DeviceBuffer(want.nbytes)
    _run(sg, sg.lib().shg_bgv_encrypt, ctx.h, out.ptr, dk.ptr, dm.ptr, ds.ptr, len(qs),
         m.shape[0], var, None)
    assert np.array_equal(out.download(want.shape), want)


@pytest.mark.gpu
@pytest.mark.parametrize("four_step_min", [13, 15])
def test_gpu_encrypt_full_size_digest(sg, oracle, four_step_min):
    """n = 2^14, six 45-bit primes: fused four-step tail and the plain one."""
    d, key, m, seeds = _encrypt_digest_inputs(oracle)
    ctx = sg.Context(d["log_n"], d["qs"], d["t"])
    sg.check(sg.lib().shg_context_set_four_step_min(ctx.h, four_step_min))
    dk, dm = sg.DeviceBuffer.from_array(key), sg.DeviceBuffer.from_array(m)
    ds = sg.DeviceBuffer.from_array(_seed_words(seeds))
    out = sg.DeviceBuffer(2 * m.nbytes)
    _run(sg, sg.lib().shg_bgv_encrypt, ctx.h, out.ptr, dk.ptr, dm.ptr, ds.ptr, 6, d["count"],
         d["variance"], None)
    assert digest(out.download((d["count"], 2, 6, 1 << 14))) == d["out_sha256"]


# --------------------------------------------------------------------------
# RNS basis conversion and BFV (reference's BFV test parameters)
# --------------------------------------------------------------------------

BFV_TAGS = sorted({k[:-len("_mul")] for k in SMALL.files
                   if k.startswith("bfv_") and k.endswith("_mul")})


def _bfv_case(tag):
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    ps = [int(p) for p in SMALL[tag + "_ps"]]
    log_n, t = (int(v) for v in SMALL[tag + "_params"])
    return log_n, qs, ps, t


@pytest.mark.parametrize("tag", BFV_TAGS)
def test_oracle_bfv_golden(oracle, tag):
    """SwitchRnsBasis, ScaleAndSwitchRnsBasis, ApproxSwitchRnsBasis,
    ModReduceMsb, ScaleAndReduceRnsBasisInPlace, ApproxModReduceLsb/Msb,
    RnsBfvCiphertext::Mul and AbsorbInPlace of the reference."""
    log_n, qs, ps, t = _bfv_case(tag)
    L, K = len(qs), len(ps)
    rns = oracle.Rns(log_n, qs + ps)
    main, aux = list(range(L)), list(range(L, L + K))
    x, y = SMALL[tag + "_x"], SMALL[tag + "_y"]
    assert np.array_equal(rns.switch_basis(main, aux, x), SMALL[tag + "_switch_up"])
    assert np.array_equal(rns.switch_basis(aux, main, y), SMALL[tag + "_switch_down"])
    assert np.array_equal(rns.switch_basis(main, aux, x, scale=True), SMALL[tag + "_scale_up"])
    assert np.array_equal(rns.approx_switch_basis(aux, main, y, True, True),
                          SMALL[tag + "_approx_down_ntt_bal"])
    assert np.array_equal(rns.approx_switch_basis(main, aux, x, False, False),
                          SMALL[tag + "_approx_up"])
    if L > 1:
        assert np.array_equal(rns.modreduce_msb(x, True), SMALL[tag + "_modreduce_msb_ntt"])
        assert np.array_equal(rns.modreduce_msb(x, False), SMALL[tag + "_modreduce_msb_coeff"])
    assert np.array_equal(rns.scale_reduce(aux, t, x, y, True, True, 0),
                          SMALL[tag + "_scale_reduce"])
    assert np.array_equal(rns.scale_reduce(aux, t, x, y, False, True, 1),
                          SMALL[tag + "_approx_lsb"])
    assert np.array_equal(rns.scale_reduce(aux, 0, x, y, True, False, 2),
                          SMALL[tag + "_approx_msb"])
    a, b = SMALL[tag + "_a"], SMALL[tag + "_b"]
    assert np.array_equal(np.stack([rns.bfv_mul(L, aux, t, a[c], b[c]) for c in range(2)]),
                          SMALL[tag + "_mul"])
    assert np.array_equal(np.stack([rns.bfv_absorb(L, aux, t, a[c], x) for c in range(2)]),
                          SMALL[tag + "_absorb"])


def _bfv_digest_inputs(oracle):
    d = DIGESTS["bfv_mul_n14_L6_K7"]
    n = 1 << d["log_n"]
    a = oracle.uniform_limbs(d["seeds"]["a"], d["qs"], n, 4).reshape(2, 2, 6, n)
    b = oracle.uniform_limbs(d["seeds"]["b"], d["qs"], n, 4).reshape(2, 2, 6, n)
    return d, a, b


def test_oracle_bfv_full_size_digest(oracle):
    d, a, b = _bfv_digest_inputs(oracle)
    rns = oracle.Rns(d["log_n"], d["qs"] + d["ps"])
    aux = list(range(6, 13))
    got = np.stack([rns.bfv_mul(6, aux, d["t"], a[c], b[c]) for c in range(2)])
    assert digest(got) == d["out_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("tag", BFV_TAGS)
def test_gpu_bfv_golden(sg, tag):
    """The device basis conversions and BFV operations against the reference."""
    log_n, qs, ps, t = _bfv_case(tag)
    L, K, n = len(qs), len(ps), 1 << log_n
    lib = sg.lib()
    ctx = sg.Context(log_n, qs, t, ps=ps)
    x, y = SMALL[tag + "_x"], SMALL[tag + "_y"]
    dx, dy = sg.DeviceBuffer.from_array(x), sg.DeviceBuffer.from_array(y)
    big = sg.DeviceBuffer(4 * 3 * max(L, K) * n * 8)

    def get(shape):
        return big.download(shape)

    _run(sg, lib.shg_poly_switch_rns_basis, ctx.h, big.ptr, dx.ptr, 0, L, 1, None)
    assert np.array_equal(get((K, n)), SMALL[tag + "_switch_up"])
    _run(sg, lib.shg_poly_switch_rns_basis, ctx.h, big.ptr, dy.ptr, 1, L, 1, None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_switch_down"])
    _run(sg, lib.shg_poly_scale_switch_rns_basis, ctx.h, big.ptr, dx.ptr, L, 1, None)
    assert np.array_equal(get((K, n)), SMALL[tag + "_scale_up"])
    _run(sg, lib.shg_poly_approx_switch_rns_basis, ctx.h, big.ptr, dy.ptr, 1, L, 1, 1, 1, None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_approx_down_ntt_bal"])
    _run(sg, lib.shg_poly_approx_switch_rns_basis, ctx.h, big.ptr, dx.ptr, 0, L, 0, 0, 1, None)
    assert np.array_equal(get((K, n)), SMALL[tag + "_approx_up"])
    if L > 1:
        ql = np.zeros(L - 1, np.uint64)
        sg.check(lib.shg_context_ql_inv(ctx.h, L - 1,
                                        ql.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
        qp = ql.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        for is_ntt, key in ((1, "_modreduce_msb_ntt"), (0, "_modreduce_msb_coeff")):
            _run(sg, lib.shg_poly_modreduce_msb, ctx.h, big.ptr, dx.ptr, qp, is_ntt, 1, L, None)
            assert np.array_equal(get((L - 1, n)), SMALL[tag + key])
    _run(sg, lib.shg_poly_scale_reduce_rns_basis, ctx.h, big.ptr, dx.ptr, dy.ptr, t, 1, 1, L,
         1, None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_scale_reduce"])
    # the same with a t other than the context's (the unfolded route)
    ctx2 = sg.Context(log_n, qs, t + 2, ps=ps)
    _run(sg, lib.shg_poly_scale_reduce_rns_basis, ctx2.h, big.ptr, dx.ptr, dy.ptr, t, 1, 1, L,
         1, None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_scale_reduce"])
    _run(sg, lib.shg_poly_approx_modreduce, ctx.h, big.ptr, dx.ptr, dy.ptr, 1, t, 0, 1, L, 1,
         None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_approx_lsb"])
    _run(sg, lib.shg_poly_approx_modreduce, ctx.h, big.ptr, dx.ptr, dy.ptr, 0, 0, 1, 0, L, 1,
         None)
    assert np.array_equal(get((L, n)), SMALL[tag + "_approx_msb"])
    a, b = SMALL[tag + "_a"], SMALL[tag + "_b"]
    da, db = sg.DeviceBuffer.from_array(a), sg.DeviceBuffer.from_array(b)
    _run(sg, lib.shg_bfv_mul, ctx.h, big.ptr, da.ptr, db.ptr, 2, L, None)
    assert np.array_equal(get((2, 3, L, n)), SMALL[tag + "_mul"])
    _run(sg, lib.shg_bfv_absorb, ctx.h, big.ptr, da.ptr, dx.ptr, 2, 2, L, None)
    assert np.array_equal(get((2, 2, L, n)), SMALL[tag + "_absorb"])


@pytest.mark.gpu
def test_gpu_bfv_full_size_digest(sg, oracle):
    """BFV ct x ct at n = 2^14, six 45-bit main and seven 45-bit aux primes."""
    d, a, b = _bfv_digest_inputs(oracle)
    ctx = sg.Context(d["log_n"], d["qs"], d["t"], ps=d["ps"])
    da, db = sg.DeviceBuffer.from_array(a), sg.DeviceBuffer.from_array(b)
    out = sg.DeviceBuffer(2 * 3 * 6 * (1 << 14) * 8)
    _run(sg, sg.lib().shg_bfv_mul, ctx.h, out.ptr, da.ptr, db.ptr, 2, 6, None)
    assert digest(out.download((2, 3, 6, 1 << 14))) == d["out_sha256"]


# --------------------------------------------------------------------------
# RnsGaloisKey::Compose
# --------------------------------------------------------------------------

COMP_TAGS = sorted({k[:-len("_out_b")] for k in SMALL.files
                    if k.startswith("galcomp_") and k.endswith("_out_b")})


@pytest.mark.parametrize("tag", COMP_TAGS)
def test_oracle_galois_compose_golden(oracle, tag):
    """Compose equals the rotation of the other key's rows (b_i, a_i)."""
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    lb = [int(b) for b in SMALL[tag + "_log_bs"]]
    p1, p2, pw = (int(v) for v in SMALL[tag + "_powers"])
    rns = oracle.Rns(log_n, qs)
    kb1, ka1, kb2, ka2 = (SMALL[f"{tag}_{x}"] for x in ("kb1", "ka1", "kb2", "ka2"))
    rows = [np.stack([rns.substitute(kb2[i], p1), rns.substitute(ka2[i], p1)])
            for i in range(kb2.shape[0])]
    out = np.stack([rns.galois(r, kb1, ka1, lb) for r in rows])
    assert np.array_equal(out[:, 0], SMALL[tag + "_out_b"])
    assert np.array_equal(out[:, 1], SMALL[tag + "_out_a"])
    assert pw == (p1 * p2) % (2 << log_n)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", COMP_TAGS)
def test_gpu_galois_compose_golden(sg, tag):
    log_n = int(tag.split("_")[1])
    qs = [int(q) for q in SMALL[tag + "_qs"]]
    lb = [int(b) for b in SMALL[tag + "_log_bs"]]
    p1, p2, pw = (int(v) for v in SMALL[tag + "_powers"])
    lib = sg.lib()
    ctx = sg.Context(log_n, qs)
    k1 = sg.Key(ctx, lb, p1, SMALL[tag + "_kb1"], SMALL[tag + "_ka1"])
    k2 = sg.Key(ctx, lb, p2, SMALL[tag + "_kb2"], SMALL[tag + "_ka2"])
    h = ctypes.c_void_p()
    sg.check(lib.shg_galois_key_compose(ctx.h, k1.h, k2.h, ctypes.byref(h)))
    try:
        assert lib.shg_key_power(h.value) == pw
        want_b, want_a = SMALL[tag + "_out_b"], SMALL[tag + "_out_a"]
        got_b, got_a = np.empty_like(want_b), np.empty_like(want_a)
        p64 = ctypes.POINTER(ctypes.c_uint64)
        sg.check(lib.shg_key_components(h.value, got_b.ctypes.data_as(p64),
                                        got_a.ctypes.data_as(p64)))
        assert np.array_equal(got_b, want_b)
        assert np.array_equal(got_a, want_a)
    finally:
        lib.shg_key_destroy(h.value)


# --------------------------------------------------------------------------
# Single-modulus symmetric RLWE (symmetric_encryption.h): SymmetricRlweKey::
# Sample, Encrypt with the ChaCha PRNG, ct + ct, ct * ct, absorb, Decrypt
# --------------------------------------------------------------------------

SYM_TAGS = sorted({k[:-len("_msgs")] for k in SMALL.files
                   if k.startswith("sym_") and k.endswith("_msgs")})


def _sym_case(tag):
    q, log_t, var = (int(x) for x in SMALL[tag + "_params"])
    log_n = int(tag.split("_")[1])
    return q, log_n, (1 << log_t) + 1, var


def _sym_ops(p, ct, pts):
    """ct + ct, ct * ct and ct * pt of pairs (i, half + i), with the oracle's
    pointwise ops (symmetric_encryption.h:111-146, 214-226, 408-445)."""
    half = ct.shape[0] // 2
    lo, hi = ct[:half], ct[half:]
    s = np.stack([[p.add(lo[i, c], hi[i, c]) for c in range(2)] for i in range(half)])
    pr = np.stack([[p.mul(lo[i, 0], hi[i, 0]),
                    p.add(p.mul(lo[i, 0], hi[i, 1]), p.mul(lo[i, 1], hi[i, 0])),
                    p.mul(lo[i, 1], hi[i, 1])] for i in range(half)])
    ab = np.stack([[p.mul(lo[i, c], pts[half + i]) for c in range(2)] for i in range(half)])
    return s, pr, ab


@pytest.mark.parametrize("tag", SYM_TAGS)
def test_oracle_symmetric_golden(oracle, tag):
    """The C restatement of Sample / Encrypt / Decrypt and the ciphertext ops
    against the reference's outputs."""
    q, log_n, t, var = _sym_case(tag)
    p = oracle.Prime(q, log_n)
    s = p.sym_key_sample(var, SMALL[tag + "_key_seed"].tobytes())
    assert np.array_equal(s, SMALL[tag + "_s"])
    msgs, seeds = SMALL[tag + "_msgs"], SMALL[tag + "_seeds"]
    pts = np.stack([p.ntt_fwd(p.import_(m)) for m in msgs])
    assert np.array_equal(pts, SMALL[tag + "_pt"])
    ct = np.stack([p.sym_encrypt_prng(t, var, s, pts[i], seeds[i].tobytes())
                   for i in range(len(msgs))])
    assert np.array_equal(ct, SMALL[tag + "_ct"])
    inj = np.stack([p.sym_encrypt(t, s, SMALL[tag + "_a"][i], SMALL[tag + "_e"][i], pts[i])
                    for i in range(len(msgs))])
    assert np.array_equal(inj, SMALL[tag + "_ct"])
    assert np.array_equal(np.stack([p.sym_decrypt(t, s, c) for c in ct]), SMALL[tag + "_dec"])
    assert np.array_equal(SMALL[tag + "_dec"], msgs)
    for nm, got in zip(("sum", "prod", "absorb"), _sym_ops(p, ct, pts)):
        assert np.array_equal(got, SMALL[f"{tag}_{nm}"]), nm
        dec = np.stack([p.sym_decrypt(t, s, c) for c in got])
        assert np.array_equal(dec, SMALL[f"{tag}_dec_{nm}"]), nm


def _sym_digest_inputs(oracle):
    d = DIGESTS["sym_c1_n12_x64"]
    n, count = 1 << d["log_n"], d["count"]
    msgs = (oracle.splitmix64(7050, count * n).reshape(count, n) %
            np.uint64((1 << d["log_t"]) + 1))
    seeds = np.array([[(7 * c + 3) % 256] * 32 for c in range(count)], np.uint8)
    p = oracle.Prime(d["q"], d["log_n"])
    s = p.sym_key_sample(d["variance"], bytes([200] * 32))
    return d, p, s, msgs, seeds


def test_oracle_symmetric_full_size_digest(oracle):
    """The C1 flow: 64 messages at n = 2^12, the 59-bit prime, t = 65537."""
    d, p, s, msgs, seeds = _sym_digest_inputs(oracle)
    t = (1 << d["log_t"]) + 1
    assert digest(s) == d["s_sha256"]
    pts = np.stack([p.ntt_fwd(p.import_(m)) for m in msgs])
    assert digest(pts) == d["pt_sha256"]
    ct = np.stack([p.sym_encrypt_prng(t, d["variance"], s, pts[i], seeds[i].tobytes())
                   for i in range(d["count"])])
    assert digest(ct) == d["ct_sha256"]
    dec = np.stack([p.sym_decrypt(t, s, c) for c in ct])
    assert digest(dec) == d["dec_sha256"] and np.array_equal(dec, msgs)
    for nm, got in zip(("sum", "prod", "absorb"), _sym_ops(p, ct, pts)):
        assert digest(got) == d[nm + "_sha256"], nm
        assert digest(np.stack([p.sym_decrypt(t, s, c) for c in got])) == \
            d[f"dec_{nm}_sha256"], nm


def _gpu_sym_flow(sg, ctx, t, var, s, pts, seeds, msgs_len):
    """The symmetric flow through the C ABI: device-sampled Encrypt
    (shg_bgv_encrypt on the one-prime context: SamplePolynomialFromPrng and
    SampleFromErrorDistribution draw as RnsPolynomial::SampleUniform and
    SampleError do for one prime), ct + ct, ct * ct, absorb, Decrypt."""
    lib = sg.lib()
    count, n = pts.shape
    half = count // 2
    ds, dp = sg.DeviceBuffer.from_array(s), sg.DeviceBuffer.from_array(pts)
    dseed = sg.DeviceBuffer.from_array(_seed_words(seeds))
    ct = sg.DeviceBuffer(count * 2 * n * 8)
    _run(sg, lib.shg_bgv_encrypt, ctx.h, ct.ptr, ds.ptr, dp.ptr, dseed.ptr, 1, count, var, None)
    cts = ct.download((count, 2, n))
    lo, hi = sg.DeviceBuffer.from_array(cts[:half]), sg.DeviceBuffer.from_array(cts[half:])
    summ = sg.DeviceBuffer(half * 2 * n * 8)
    _run(sg, lib.shg_poly_add, ctx.h, summ.ptr, lo.ptr, hi.ptr, 2 * half, 1, None)
    prod = sg.DeviceBuffer(half * 3 * n * 8)
    _run(sg, lib.shg_ct_tensor, ctx.h, prod.ptr, lo.ptr, hi.ptr, half, 1, None)
    pt2 = sg.DeviceBuffer.from_array(np.repeat(pts[half:], 2, axis=0))
    ab = sg.DeviceBuffer(half * 2 * n * 8)
    _run(sg, lib.shg_poly_mul, ctx.h, ab.ptr, lo.ptr, pt2.ptr, 2 * half, 1, None)
    out = {"ct": cts, "sum": summ.download((half, 2, n)), "prod": prod.download((half, 3, n)),
           "absorb": ab.download((half, 2, n))}
    dec = sg.DeviceBuffer(count * n * 8)
    for nm, buf, ln, c in (("dec", ct, 2, count), ("dec_sum", summ, 2, half),
                           ("dec_prod", prod, 3, half), ("dec_absorb", ab, 2, half)):
        _run(sg, lib.shg_symmetric_decrypt, ctx.h, dec.ptr, ds.ptr, buf.ptr, ln, c, None)
        out[nm] = dec.download((c, n))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("tag", SYM_TAGS)
def test_gpu_symmetric_golden(sg, oracle, tag):
    """Device Encrypt (injected randomness and device-sampled), the
    ciphertext ops and Decrypt against the reference's outputs."""
    q, log_n, t, var = _sym_case(tag)
    n = 1 << log_n
    msgs = SMALL[tag + "_msgs"]
    count = len(msgs)
    ctx = sg.Context(log_n, [q], t)
    s, pts = SMALL[tag + "_s"], SMALL[tag + "_pt"]
    # the plaintexts' NTT on the device
    dp = sg.DeviceBuffer.from_array(oracle.Prime(q, log_n).import_(msgs.reshape(-1))
                                    .reshape(count, n))
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, dp.ptr, count, 1, None)
    assert np.array_equal(dp.download((count, n)), pts)
    # internal::Encrypt with the reference's own a and e
    ds = sg.DeviceBuffer.from_array(s)
    da, de = sg.DeviceBuffer.from_array(SMALL[tag + "_a"]), sg.DeviceBuffer.from_array(
        SMALL[tag + "_e"])
    ct = sg.DeviceBuffer(count * 2 * n * 8)
    _run(sg, sg.lib().shg_symmetric_encrypt, ctx.h, ct.ptr, ds.ptr, da.ptr, de.ptr, dp.ptr,
         count, None)
    assert np.array_equal(ct.download((count, 2, n)), SMALL[tag + "_ct"])
    got = _gpu_sym_flow(sg, ctx, t, var, s, pts, SMALL[tag + "_seeds"], count)
    for nm, v in got.items():
        assert np.array_equal(v, SMALL[f"{tag}_{nm}"]), nm


@pytest.mark.gpu
def test_gpu_symmetric_full_size_digest(sg, oracle):
    """C1 on the device: 64 messages at n = 2^12, q = 576460752303415297,
    t = 65537 -- Encrypt with on-device ChaCha sampling, ct + ct, ct * ct,
    absorb, Decrypt, every output's digest equal to the reference's."""
    d, p, s, msgs, seeds = _sym_digest_inputs(oracle)
    assert digest(s) == d["s_sha256"]
    n, count = 1 << d["log_n"], d["count"]
    ctx = sg.Context(d["log_n"], [d["q"]], (1 << d["log_t"]) + 1)
    dp = sg.DeviceBuffer.from_array(p.import_(msgs.reshape(-1)).reshape(count, n))
    _run(sg, sg.lib().shg_ntt_forward, ctx.h, dp.ptr, count, 1, None)
    pts = dp.download((count, n))
    assert digest(pts) == d["pt_sha256"]
    got = _gpu_sym_flow(sg, ctx, (1 << d["log_t"]) + 1, d["variance"], s, pts, seeds, count)
    for nm, v in got.items():
        assert digest(v) == d[nm + "_sha256"], nm
    assert np.array_equal(got["dec"], msgs)
