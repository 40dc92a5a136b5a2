"""The faster CPU gate bootstrap timed beside the oracle in bench.py
(oracle/tfhe_cpu_fast.cpp: the N/2-point twisted transform of the upstream
library's method, FP64).  It is a timed comparison, not a checker, so it
is checked here against the oracle: the same decrypted gate outputs, and on
the default set phases within the small-batch tolerance the engine's tests
use (the two FFTs round differently, which moves a gadget digit now and
then and so gives each output its own noise)."""
import numpy as np
import pytest

from oracle import pyoracle
from tests.helpers import wrap_diff

PHASE_TOL = 2 ** 26  # 2^-6 of a turn


@pytest.mark.parametrize("params", ["default", "stress"])
def test_fast_cpu_gates_decrypt_like_the_oracle(oracle, params):
    P = pyoracle.default_params() if params == "default" else pyoracle.stress_params()
    lwe, _, ks, bk = oracle.gate_keyset(P, [3])
    bk_fft = oracle.bk_to_fft(P, bk)
    fast = pyoracle.CpuFast(P, bk, ks)
    try:
        rng = np.random.default_rng(11)
        count = 20
        a, b = rng.integers(0, 2, count), rng.integers(0, 2, count)
        gates = np.arange(count, dtype=np.int32) % 10  # every gate type twice
        oracle.set_seed([11])
        ca, cb = oracle.encrypt_bits(P, a, lwe), oracle.encrypt_bits(P, b, lwe)
        ref = oracle.boots_gate_batch(P, bk_fft, ks, gates, ca, cb)
        got = fast.boots_gates(gates, ca, cb)
        truth = np.array([pyoracle.GATE_FN[name](x, y) for name, x, y in
                          zip([list(pyoracle.GATES)[g] for g in gates], a, b)])
        assert (oracle.decrypt_bits(P, got, lwe) == truth).all()
        assert (oracle.decrypt_bits(P, ref, lwe) == truth).all()
        if params == "default":
            d = wrap_diff(oracle.phases(got, lwe, P.n), oracle.phases(ref, lwe, P.n))
            assert np.abs(d).max() <= PHASE_TOL
    finally:
        fast.close()


def test_fast_cpu_refuses_bad_parameters():
    P = pyoracle.default_params()
    P.N = 1000  # not a power of two
    with pytest.raises(ValueError):
        pyoracle.CpuFast(P, np.zeros(4, np.int32), np.zeros(4, np.int32))
