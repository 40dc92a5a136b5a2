"""Small helpers shared by the tests."""
import numpy as np


def wrap_diff(a, b):
    """Signed difference mod 2^32 of int32 arrays."""
    d = np.asarray(a, np.int64) - np.asarray(b, np.int64)
    return (d + 2 ** 31) % 2 ** 32 - 2 ** 31


def negacyclic_mul(a, b):
    """Exact negacyclic product of two integer polynomials (int64 result,
    not reduced)."""
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    N = len(a)
    r = np.zeros(N, np.int64)
    for j in np.nonzero(a)[0]:
        r[j:] += a[j] * b[:N - j]
        r[:j] -= a[j] * b[N - j:]
    return r


def mod_switch_from_torus32_ref(phase, msize):
    """numeric-functions.cpp:59-65 restated on Python integers."""
    interv = ((1 << 63) // msize) * 2
    half = interv // 2
    phase64 = (((int(phase) & 0xFFFFFFFF) << 32) + half) % (1 << 64)
    return phase64 // interv


def mod_switch_to_torus32_ref(mu, msize):
    """numeric-functions.cpp:71-76 restated on Python integers."""
    interv = ((1 << 63) // msize) * 2
    phase64 = (mu * interv) % (1 << 64)
    v = phase64 >> 32
    return v - (1 << 32) if v >= (1 << 31) else v


def tlwe_phase(acc, tlwe_key, N, k=1):
    """Phase b - sum_i a_i s_i (negacyclic) of TLWE samples (..., (k+1) N)."""
    acc = np.asarray(acc, np.int64).reshape(-1, (k + 1) * N)
    key = np.asarray(tlwe_key, np.int64).reshape(k, N)
    out = np.empty((acc.shape[0], N), np.int64)
    for c in range(acc.shape[0]):
        ph = acc[c, k * N:].copy()
        for i in range(k):
            ph -= negacyclic_mul(key[i], acc[c, i * N:(i + 1) * N])
        out[c] = ph
    return ((out + 2 ** 31) % 2 ** 32 - 2 ** 31).astype(np.int64)
