"""Generate tests/golden/golden_default.npz from the CPU oracle.

The reference ships no golden vectors; these are produced by the oracle
(itself pinned against the reference's own code, tests/test_oracle_vs_
reference.py) from fixed seeds, so later runs -- on this machine, on the GPU
machine, after refactors -- can be checked against them:

  keys         seed [0], default set: SHA-256 of the LWE key, TLWE key,
               key-switching key and bootstrapping key (not stored)
  gates        8 gates (one of each of the first 8 gate ids) on inputs
               encrypted from seed [1]; outputs of the oracle (FP64 path)
  extprod      one external product: TLWE from numpy seed 2, TGSW of X^e
               (e from seed 3) under the seed-0 TLWE key; exact int64 result
  keyswitch    one key switch of a random extracted sample with the seed-0
               key-switching key
  modswitch    1000 values and their modSwitchFromTorus32(., 2048)

    python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "golden_default.npz")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def make():
    o = pyoracle.get()
    P = pyoracle.default_params()
    lwe, tlwe, ks, bk = o.gate_keyset(P, [0])
    bk_fft = o.bk_to_fft(P, bk)
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2, 8)
    b = rng.integers(0, 2, 8)
    gates = np.arange(8, dtype=np.int32)
    o.set_seed([1])
    ca = o.encrypt_bits(P, a, lwe)
    cb = o.encrypt_bits(P, b, lwe)
    out = o.boots_gate_batch(P, bk_fft, ks, gates, ca, cb)
    # external product
    r2 = np.random.default_rng(2)
    acc = r2.integers(-2 ** 31, 2 ** 31, 2 * P.N).astype(np.int32)
    e = int(np.random.default_rng(3).integers(0, 2 * P.N))
    o.set_seed([3])
    g = o.tgsw_encrypt_int(P, 1, P.tlwe_alpha, tlwe).reshape(P.kpl, 2, P.N)
    g = np.stack([[o.mul_by_xai(P.N, e, g[p, j]) for j in range(2)] for p in range(P.kpl)]).reshape(-1)
    ep = o.extern_mul_exact(P, acc, g)
    # key switch
    u = np.random.default_rng(4).integers(-2 ** 31, 2 ** 31, P.N + 1).astype(np.int32)
    ksout = o.keyswitch(P, ks, u)
    ms_in = np.random.default_rng(5).integers(-2 ** 31, 2 ** 31, 1000).astype(np.int32)
    ms_out = np.array([o.mod_switch_from_torus32(int(v), 2048) for v in ms_in], np.int32)
    np.savez_compressed(
        OUT, key_sha=np.array([sha(lwe), sha(tlwe), sha(ks), sha(bk)]),
        gate_bits_a=a, gate_bits_b=b, gate_ids=gates, gate_ca=ca, gate_cb=cb, gate_out=out,
        ep_acc=acc, ep_gsw=g, ep_e=np.array([e]), ep_exact=ep,
        ks_in=u, ks_out=ksout, ms_in=ms_in, ms_out=ms_out)
    return OUT


if __name__ == "__main__":
    print(make())
