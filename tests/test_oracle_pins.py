"""Pins of the CPU oracle against what the reference itself fixes.

The reference ships no golden vectors (its .gitignore drops keys/data/logs and
its testbenches compare live against the absent upstream library).  What it
does fix, and what is checked here:
  * constants: mu = modSwitchToTorus32(1, 8) = 2^29 (tb:267), the gadget
    offset 2164391936 (constants.h:24);
  * exact integer semantics of modSwitchFromTorus32/ToTorus32
    (numeric-functions.cpp:59-76), decomposition (tGswFFTExternMulToTLwe.cpp:
    76-95), X^a and X^a - 1 rotations (mulByXaiOrCopy.cpp:25-41,
    tfhe_MuxRotate_FFT.cpp:5-24), key switching (lwe-keyswitch-functions.cpp:
    114-129);
  * the Lagrange convention (values at w^(2m+1), tGswFFTExternMulToTLwe.cpp:
    97-130) and the truncating conversion back (TorusPolynomial_fft.cpp:4-43);
  * the end-to-end known answer of test_bench/: 499 OR 388 = 503 with the
    seed {314, 1592, 657} (alice.c:13-15, cloud.c:33-36, verify.c:31).
"""
import numpy as np
import pytest

from helpers import (mod_switch_from_torus32_ref, mod_switch_to_torus32_ref, negacyclic_mul,
                     tlwe_phase, wrap_diff)
from oracle import pyoracle


def test_mu_and_offset(oracle, P):
    assert oracle.mod_switch_to_torus32(1, 8) == 2 ** 29
    assert oracle.mod_switch_to_torus32(-1, 8) == -(2 ** 29)
    assert oracle.mod_switch_to_torus32(1, 4) == 2 ** 30
    # offset: decompose(0) gives digit -halfBg + (offset bits) -> check via value
    d = oracle.decompose(P, np.zeros(P.N, np.int32))
    # 0 + 2164391936 = 0x81020000: digits 0x40,0x40,0x40 -> each 64 - 64 = 0
    assert (d == 0).all()
    off = sum(64 * (1 << (32 - (i + 1) * 7)) for i in range(3))
    assert off == 2164391936


def test_mod_switch_semantics(oracle):
    rng = np.random.default_rng(11)
    vals = list(rng.integers(-2 ** 31, 2 ** 31, 2000)) + [0, -1, 2 ** 31 - 1, -2 ** 31, 2 ** 20, 2 ** 20 - 1]
    for msize in (2048, 1024, 8, 4):
        for v in vals:
            assert oracle.mod_switch_from_torus32(int(v), msize) == mod_switch_from_torus32_ref(v, msize)
    for mu in range(-9, 10):
        for msize in (8, 4, 2048):
            assert oracle.mod_switch_to_torus32(mu, msize) == mod_switch_to_torus32_ref(mu, msize)


def test_decomposition_reconstructs(oracle):
    rng = np.random.default_rng(12)
    for Pm in (pyoracle.default_params(), pyoracle.stress_params()):
        x = rng.integers(-2 ** 31, 2 ** 31, Pm.N).astype(np.int32)
        d = oracle.decompose(Pm, x)
        half = 1 << (Pm.Bgbit - 1)
        assert d.min() >= -half and d.max() < half
        rec = sum(d[p].astype(np.int64) << (32 - (p + 1) * Pm.Bgbit) for p in range(Pm.l))
        err = wrap_diff(rec, x)
        # truncation of the bits below l*Bgbit (no rounding term in the offset)
        lost = 1 << (32 - Pm.l * Pm.Bgbit)
        assert err.max() <= 0 and err.min() > -lost


def test_rotations(oracle, P):
    rng = np.random.default_rng(13)
    N = P.N
    x = rng.integers(-2 ** 31, 2 ** 31, N).astype(np.int32)
    for a in (0, 1, 5, N - 1, N, N + 3, 2 * N - 1):
        mono = np.zeros(N, np.int64)
        if a < N:
            mono[a] = 1
        else:
            mono[a - N] = -1
        want = negacyclic_mul(mono, x)
        got = oracle.mul_by_xai(N, a, x)
        assert (wrap_diff(got, want) == 0).all()
        got1 = oracle.mul_by_xai_minus_one(N, a, x)
        assert (wrap_diff(got1, want - x.astype(np.int64)) == 0).all()


def test_lagrange_convention(oracle, P):
    """IntPolynomial -> Lagrange gives P(w^(2m+1)), w = e^{i pi/N}."""
    rng = np.random.default_rng(14)
    N = P.N
    c = rng.integers(-64, 64, N).astype(np.int32)
    got = oracle.int_poly_ifft(N, c)
    w = np.exp(1j * np.pi * (2 * np.arange(N // 2) + 1) / N)
    want = np.array([np.polyval(c[::-1].astype(np.float64), wi) for wi in w])
    assert np.allclose(got, want, rtol=0, atol=1e-7 * np.abs(want).max())
    # torus round trip: fft(ifft(t)) reproduces t up to the truncation
    t = rng.integers(-2 ** 31, 2 ** 31, N).astype(np.int32)
    back = oracle.torus_poly_fft(N, oracle.torus_poly_ifft(N, t))
    assert np.abs(wrap_diff(back, t)).max() <= 1


def test_external_product_fft_vs_exact(oracle, P):
    rng = np.random.default_rng(15)
    tlwe_key = rng.integers(0, 2, P.N).astype(np.int32)
    oracle.set_seed([3])
    for e in (0, 1, 700, 2047):
        # TGSW encryption of X^e (message as a monomial): encrypt 1, rotate rows
        g = oracle.tgsw_encrypt_int(P, 1, P.tlwe_alpha, tlwe_key).reshape(P.kpl, P.k + 1, P.N)
        g = np.stack([[oracle.mul_by_xai(P.N, e, g[p, j]) for j in range(P.k + 1)]
                      for p in range(P.kpl)]).reshape(-1)
        acc = rng.integers(-2 ** 31, 2 ** 31, (P.k + 1) * P.N).astype(np.int32)
        exact = oracle.extern_mul_exact(P, acc, g)
        fft = oracle.extern_mul_fft(P, acc, oracle.tgsw_to_fft(P, g))
        assert np.abs(wrap_diff(fft, exact)).max() <= 2


def test_keyswitch_phase(oracle, P, keys):
    """KS(u) decrypts under the LWE key to the phase of u under the
    extracted TLWE key, up to the key-switch noise and precision."""
    rng = np.random.default_rng(16)
    nk = P.k * P.N
    o = oracle
    for _ in range(4):
        mu = int(rng.choice([2 ** 29, -(2 ** 29)]))
        u = np.zeros(nk + 1, np.int32)
        o.lib.orc_lwe_encrypt(u.ctypes.data_as(pyoracle.I32P), mu, 2.0 ** -20,
                              keys["tlwe"].ctypes.data_as(pyoracle.I32P), nk)
        out = o.keyswitch(P, keys["ks"], u)
        ph_in = o.phases(u, keys["tlwe"], nk)[0]
        ph_out = o.phases(out, keys["lwe"], P.n)[0]
        assert abs(int(wrap_diff(ph_out, ph_in))) < 2 ** 32 * 0.02


def test_known_answer_499_or_388(oracle, P):
    """test_bench/: alice encrypts 499 and 388 bit by bit (seed
    {314,1592,657}), the cloud ORs 16 bits, verify decrypts 499 | 388."""
    lwe, tlwe, ks, bk = oracle.gate_keyset(P, [314, 1592, 657])
    bk_fft = oracle.bk_to_fft(P, bk)
    c1 = oracle.encrypt_bits(P, [(499 >> i) & 1 for i in range(16)], lwe)
    c2 = oracle.encrypt_bits(P, [(388 >> i) & 1 for i in range(16)], lwe)
    out = oracle.boots_gate_batch(P, bk_fft, ks, [pyoracle.GATES["OR"]] * 16, c1, c2)
    bits = oracle.decrypt_bits(P, out, lwe)
    assert sum(int(b) << i for i, b in enumerate(bits)) == (499 | 388) == 503


@pytest.mark.parametrize("gate", sorted(pyoracle.GATES))
def test_gate_truth_tables(oracle, P, keys, gate):
    oracle.set_seed([21])
    a = np.array([0, 0, 1, 1])
    b = np.array([0, 1, 0, 1])
    ca = oracle.encrypt_bits(P, a, keys["lwe"])
    cb = oracle.encrypt_bits(P, b, keys["lwe"])
    out = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], [pyoracle.GATES[gate]] * 4, ca, cb)
    got = oracle.decrypt_bits(P, out, keys["lwe"])
    want = np.array([pyoracle.GATE_FN[gate](x, y) for x, y in zip(a, b)])
    assert (got == want).all()


def test_mux_truth_table(oracle, P, keys):
    oracle.set_seed([22])
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                ca, cb, cc = oracle.encrypt_bits(P, [a, b, c], keys["lwe"])
                out = oracle.boots_mux(P, keys["bk_fft"], keys["ks"], ca, cb, cc)
                assert oracle.decrypt_bits(P, out, keys["lwe"])[0] == (b if a else c)


def test_mux_batch_is_the_single_mux(oracle, P, keys):
    """The threaded bootsMUX batch gives, word for word, the single call's
    results (same code per item, any thread)."""
    oracle.set_seed([23])
    a, b, c = (oracle.encrypt_bits(P, bits, keys["lwe"]) for bits in ([1, 0, 1], [0, 1, 1], [1, 1, 0]))
    got = oracle.boots_mux_batch(P, keys["bk_fft"], keys["ks"], a, b, c)
    for i in range(3):
        assert (got[i] == oracle.boots_mux(P, keys["bk_fft"], keys["ks"], a[i], b[i], c[i])).all()


def test_blind_rotate_fft_vs_exact_small_n(oracle):
    """Full blind rotation, FP64 transform against the exact integer product,
    on a shortened LWE dimension so that the exact path is quick.  Compared
    by TLWE phase: a one-unit rounding difference can move a gadget digit
    across its boundary, which adds a different key row (a fresh mask); from
    then on the two accumulators carry independent noise terms, so their
    phases agree to the bootstrapping-noise level, not to the rounding level."""
    Ps = pyoracle.default_params()
    Ps.n = 12
    rng = np.random.default_rng(17)
    tlwe_key = rng.integers(0, 2, Ps.N).astype(np.int32)
    lwe_key = rng.integers(0, 2, Ps.n).astype(np.int32)
    oracle.set_seed([4])
    bk = np.concatenate([oracle.tgsw_encrypt_int(Ps, int(s), Ps.tlwe_alpha, tlwe_key) for s in lwe_key])
    bk_fft = oracle.bk_to_fft(Ps, bk)
    x = rng.integers(-2 ** 31, 2 ** 31, Ps.n + 1).astype(np.int32)
    bara, acc0 = oracle.bootstrap_prologue(Ps, 2 ** 29, x)
    a = oracle.blind_rotate_fft(Ps, acc0, bk_fft, bara)
    b = oracle.blind_rotate_exact(Ps, acc0, bk, bara)
    d = wrap_diff(tlwe_phase(a, tlwe_key, Ps.N), tlwe_phase(b, tlwe_key, Ps.N))
    assert np.abs(d).max() <= 2 ** 25
    # and the phase is the rotated test vector: +-mu up to the noise
    ph = tlwe_phase(b, tlwe_key, Ps.N)
    assert np.abs(np.abs(ph) - 2 ** 29).max() < 2 ** 24
