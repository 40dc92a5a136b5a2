"""The oracle against the reference's own code (oracle/_ref, built from the
reference's sources by oracle/ref_pin/build_ref.py).  CPU only; skipped where
the reference sources are not present (no reference checkout on the machine).

What is pinned, and how tightly:
  * numeric-functions.cpp (RNG, gaussian32, dtot32, modSwitch, approxPhase):
    bit-exact, same seeds give the same streams;
  * lwe-functions.cpp (lweKeyGen, lweSymEncrypt, lwePhase, the OR
    combination of tfhe_blindRotate_FFT_tb.cpp:271-276): bit-exact;
  * lwe-keyswitch-functions.cpp (lweCreateKeySwitchKey, lweKeySwitch):
    bit-exact;
  * decompose / tGswTorus32PolynomialDecompH: bit-exact;
  * the bootstrap front end (tfhe_bootstrap_woKS_FFT.cpp + mulByXaiOrCopy.cpp):
    bit-exact;
  * Int -> Lagrange (the reference's `ifft` over its SPIRAL Pease FFT):
    relative 1e-12; Lagrange -> Torus32: 1 unit;
  * tGswFFTExternMulToTLwe_FPGA and tfhe_MuxRotate_FFT_FPGA: 2 units;
  * the blind rotation of the reference's MuxRotate over several steps: by
    phase (the digit-boundary effect, see test_oracle_pins);
  * the shipped tfhe_blindRotate_FFT: exactly one MuxRotate step (its loop
    bound, tfhe_blindRotate_FFT.cpp:112).
"""
import numpy as np
import pytest

from helpers import tlwe_phase, wrap_diff
from oracle import pyoracle
from oracle.ref_pin import pyref

pytestmark = pytest.mark.skipif(not pyref.available(), reason="reference sources not present")


@pytest.fixture(scope="module")
def ref():
    return pyref.get()


def test_reference_parameters(ref, P):
    assert (ref.n, ref.N, ref.k, ref.l, ref.Bgbit, ref.ks_t, ref.ks_basebit) == \
        (P.n, P.N, P.k, P.l, P.Bgbit, P.ks_t, P.ks_basebit)


def test_numeric_functions(ref, oracle):
    rng = np.random.default_rng(51)
    for v in rng.integers(-2 ** 31, 2 ** 31, 500):
        for m in (2048, 8, 4):
            assert ref.tfhe.modSwitchFromTorus32(int(v), m) == oracle.mod_switch_from_torus32(int(v), m)
            assert ref.tfhe.approxPhase(int(v), m) == oracle.approx_phase(int(v), m)
    for mu in range(-5, 6):
        assert ref.tfhe.modSwitchToTorus32(mu, 8) == oracle.mod_switch_to_torus32(mu, 8)
    for d in rng.standard_normal(200) * 3:
        assert ref.tfhe.dtot32(float(d)) == oracle.dtot32(float(d))
    ref.set_seed([9, 8, 7])
    oracle.set_seed([9, 8, 7])
    a = [ref.tfhe.gaussian32(123, 2.0 ** -15) for _ in range(300)]
    b = [oracle.gaussian32(123, 2.0 ** -15) for _ in range(300)]
    assert a == b


def test_lwe_keygen_and_encryption(ref, oracle, P):
    ref.set_seed([314, 1592, 657])
    oracle.set_seed([314, 1592, 657])
    k1 = ref.lwe_keygen(P.n)
    k2 = np.zeros(P.n, np.int32)
    oracle.lib.orc_lwe_keygen(k2.ctypes.data_as(pyoracle.I32P), P.n)
    assert (k1 == k2).all()
    for mu in (2 ** 29, -(2 ** 29), 0):
        c1 = ref.lwe_encrypt(k1, mu, P.lwe_alpha)
        c2 = np.zeros(P.n + 1, np.int32)
        oracle.lib.orc_lwe_encrypt(c2.ctypes.data_as(pyoracle.I32P), mu, P.lwe_alpha,
                                   k2.ctypes.data_as(pyoracle.I32P), P.n)
        assert (c1 == c2).all()
        assert ref.tfhe.refu_lwe_phase(P.n, pyref._p(k1, pyref.I32P), pyref._p(c1, pyref.I32P)) == \
            oracle.phases(c2, k2, P.n)[0]


def test_keyswitch_key_and_keyswitch(ref, oracle, P):
    """lweCreateKeySwitchKey from the same seed, then lweKeySwitch."""
    rng = np.random.default_rng(52)
    in_key = rng.integers(0, 2, P.k * P.N).astype(np.int32)
    out_key = rng.integers(0, 2, P.n).astype(np.int32)
    ref.set_seed([77])
    t1 = ref.create_ks_key(in_key, out_key, P.ks_t, P.ks_basebit, P.lwe_alpha)
    oracle.set_seed([77])
    t2 = np.zeros(P.ks_words(), np.int32)
    oracle.lib.orc_create_ks_key(pyoracle.ctypes.byref(P), t2.ctypes.data_as(pyoracle.I32P),
                                 in_key.ctypes.data_as(pyoracle.I32P), P.k * P.N,
                                 out_key.ctypes.data_as(pyoracle.I32P))
    assert (t1 == t2).all()
    for _ in range(3):
        u = rng.integers(-2 ** 31, 2 ** 31, P.k * P.N + 1).astype(np.int32)
        a = ref.keyswitch(t1, u, P.k * P.N, P.n, P.ks_t, P.ks_basebit)
        b = oracle.keyswitch(P, t2, u)
        assert (a == b).all()


def test_gate_combination_or(ref, oracle, P):
    rng = np.random.default_rng(53)
    ca = rng.integers(-2 ** 31, 2 ** 31, P.n + 1).astype(np.int32)
    cb = rng.integers(-2 ** 31, 2 ** 31, P.n + 1).astype(np.int32)
    a = ref.or_combination(oracle.mod_switch_to_torus32(1, 8), ca, cb)
    assert (a == oracle.gate_combine(P, "OR", ca, cb)).all()


def test_decomposition(ref, oracle, P):
    rng = np.random.default_rng(54)
    for _ in range(4):
        x = rng.integers(-2 ** 31, 2 ** 31, P.N).astype(np.int32)
        want = oracle.decompose(P, x)
        assert (ref.decompose(x) == want).all()
        assert (ref.decomp_h(x) == want).all()


def test_lagrange_transforms(ref, oracle, P):
    rng = np.random.default_rng(55)
    d = rng.integers(-64, 64, P.N).astype(np.int32)
    a, b = ref.int_ifft(d), oracle.int_poly_ifft(P.N, d)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    t = rng.integers(-2 ** 31, 2 ** 31, P.N).astype(np.int32)
    lag = oracle.torus_poly_ifft(P.N, t)
    assert np.abs(wrap_diff(ref.torus_fft(lag), oracle.torus_poly_fft(P.N, lag))).max() <= 1


def _tgsw(oracle, P, bit, seed, key):
    oracle.set_seed([seed])
    g = oracle.tgsw_encrypt_int(P, bit, P.tlwe_alpha, key)
    return g, oracle.tgsw_to_fft(P, g)


def test_external_product_and_mux_rotate(ref, oracle, P):
    rng = np.random.default_rng(56)
    key = rng.integers(0, 2, P.N).astype(np.int32)
    g, gf = _tgsw(oracle, P, 1, 57, key)
    for a in (0, 1, 700, 1024, 2047):
        acc = rng.integers(-2 ** 31, 2 ** 31, 2 * P.N).astype(np.int32)
        re = ref.extern_mul(acc, gf)
        assert np.abs(wrap_diff(re, oracle.extern_mul_fft(P, acc, gf))).max() <= 2
        assert np.abs(wrap_diff(re, oracle.extern_mul_exact(P, acc, g))).max() <= 2
        if a:
            rm = ref.mux_rotate(acc, gf, a)
            assert np.abs(wrap_diff(rm, oracle.mux_rotate_fft(P, acc, gf, a))).max() <= 2


def test_bootstrap_front_end(ref, oracle, P):
    rng = np.random.default_rng(58)
    for _ in range(4):
        x = rng.integers(-2 ** 31, 2 ** 31, P.n + 1).astype(np.int32)
        tv, bara, barb, rot = ref.bootstrap_front(x, 2 ** 29)
        obara, oacc = oracle.bootstrap_prologue(P, 2 ** 29, x)
        assert (tv == 2 ** 29).all()
        assert (bara == obara).all()
        assert barb == oracle.mod_switch_from_torus32(int(x[P.n]), 2 * P.N)
        assert (rot == oacc[P.N:]).all() and (oacc[:P.N] == 0).all()


def test_blind_rotation_steps(ref, oracle, P):
    """The reference's MuxRotate chained over several steps (the loop its
    blindRotate kernel means to run) against the oracle's blind rotation."""
    rng = np.random.default_rng(59)
    key = rng.integers(0, 2, P.N).astype(np.int32)
    steps = 5
    lwe_bits = rng.integers(0, 2, steps)
    pairs = [_tgsw(oracle, P, int(b), 60 + i, key) for i, b in enumerate(lwe_bits)]
    bk_fft = np.concatenate([gf for _, gf in pairs])
    bara = np.array([3, 0, 1500, 2047, 1024], np.int32)
    acc0 = np.zeros(2 * P.N, np.int32)
    acc0[P.N:] = 2 ** 29
    Ps = pyoracle.default_params()
    Ps.n = steps
    a = ref.blind_rotate(acc0, bk_fft, bara)
    b = oracle.blind_rotate_fft(Ps, acc0, bk_fft, bara)
    d = wrap_diff(tlwe_phase(a, key, P.N), tlwe_phase(b, key, P.N))
    assert np.abs(d).max() <= 2 ** 24  # noise level; a wrong step shows at 2^29


def test_shipped_blind_rotate_runs_one_step(ref, oracle, P):
    """tfhe_blindRotate_FFT as shipped stops after step 0
    (tfhe_blindRotate_FFT.cpp:112): equal to one MuxRotate."""
    rng = np.random.default_rng(61)
    key = rng.integers(0, 2, P.N).astype(np.int32)
    _, gf = _tgsw(oracle, P, 1, 62, key)
    acc = rng.integers(-2 ** 31, 2 ** 31, 2 * P.N).astype(np.int32)
    bara = rng.integers(1, 2 * P.N, P.n).astype(np.int32)
    shipped = ref.blind_rotate_shipped(acc, gf, bara)
    one = oracle.mux_rotate_fft(P, acc, gf, int(bara[0]))
    assert np.abs(wrap_diff(shipped, one)).max() <= 2
