"""CPU-side checks of the C ABI library: it loads, exports every function
declared in include/*.h, its host-side client code (keygen, encryption,
decryption) reproduces the oracle bit for bit, and argument checking returns
status codes instead of exiting -- all without launching a kernel."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            name = m.group(1)
            if name.startswith(("tfhe_gpu_", "tfhe_client_", "tfhe_keyfile_")) and name not in ("tfhe_gpu_status",):
                names.add(name)
    return sorted(names)


def compat_functions():
    """Functions declared by the upstream-API headers include/tfhe/*.h."""
    names = set()
    inc = os.path.join(ROOT, "include", "tfhe")
    for f in sorted(os.listdir(inc)):
        text = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            if m.group(1) not in ("defined",):
                names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("tfhe_gpu_create", "tfhe_gpu_tGswFFTExternMulToTLwe", "tfhe_gpu_tfhe_blindRotate_FFT",
                 "tfhe_gpu_tfhe_MuxRotate_FFT", "tfhe_gpu_lweKeySwitch", "tfhe_gpu_bootsGate",
                 "tfhe_gpu_IntPolynomial_ifft", "tfhe_gpu_TorusPolynomial_fft",
                 "tfhe_gpu_tLweExtractLweSample", "tfhe_gpu_tLweMulByXaiMinusOne"):
        assert must in names


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the binding knows a signature for each of them
    assert set(declared_functions()) <= set(pkg.SIGNATURES)


def test_library_exports_upstream_api(pkg):
    names = compat_functions()
    for must in ("bootsNAND", "bootsOR", "bootsAND", "bootsXOR", "bootsXNOR", "bootsMUX", "bootsCONSTANT",
                 "new_tfheGateBootstrappingCloudKeySet_fromFile", "import_gate_bootstrapping_ciphertext_fromFile",
                 "new_random_gate_bootstrapping_secret_keyset", "bootsSymEncrypt", "bootsSymDecrypt"):
        assert must in names
    lib = pkg.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_client_keygen_matches_oracle(pkg, oracle, keys):
    P = pkg.default_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    assert (lwe == keys["lwe"]).all()
    assert (tlwe == keys["tlwe"]).all()
    assert (ks == keys["ks"]).all()
    assert (bk == keys["bk"]).all()


def test_client_encrypt_decrypt_matches_oracle(pkg, oracle, keys):
    P = pkg.default_params()
    OP = pyoracle.default_params()
    bits = np.array([1, 0, 0, 1, 1, 1, 0, 0])
    pkg.set_seed([7])
    a = pkg.encrypt_bits(P, bits, keys["lwe"])
    oracle.set_seed([7])
    b = oracle.encrypt_bits(OP, bits, keys["lwe"])
    assert (a == b).all()
    assert (pkg.decrypt_bits(P, a, keys["lwe"]) == bits).all()
    assert (pkg.phases(a, keys["lwe"]) == oracle.phases(b, keys["lwe"], OP.n)).all()
    assert pkg.lib().tfhe_client_mod_switch_to_torus32(1, 8) == 2 ** 29


def test_stress_set_keygen_matches_oracle(pkg, oracle):
    P = pkg.stress_params()
    OP = pyoracle.stress_params()
    a = pkg.gate_keyset(P, [5])
    b = oracle.gate_keyset(OP, [5])
    for x, y in zip(a, b):
        assert (x == y).all()


def test_create_rejects_bad_params_without_gpu(pkg):
    lib = pkg.lib()
    h = ctypes.c_void_p()
    for field, value in (("N", 2048), ("k", 2), ("Bgbit", 0), ("ks_basebit", 3), ("ks_t", 6),
                         ("l", 4), ("split_bits", 40)):
        P = pkg.default_params()
        setattr(P, field, value)
        assert lib.tfhe_gpu_create(ctypes.byref(P), 0, ctypes.byref(h)) == 1  # BAD_PARAM
        assert not h.value
    assert lib.tfhe_gpu_create(None, 0, ctypes.byref(h)) == 1


def test_status_strings_and_null_context(pkg):
    lib = pkg.lib()
    assert lib.tfhe_gpu_status_string(0) == b"ok"
    assert lib.tfhe_gpu_status_string(5) == b"key not uploaded"
    assert lib.tfhe_gpu_last_error(None) == b"null context"
    assert lib.tfhe_gpu_synchronize(None) == 1
    assert lib.tfhe_gpu_bootsGate(None, 0, None, None, None, 1, 0, None) == 1
    lib.tfhe_gpu_destroy(None)  # no-op


def test_client_rejects_bad_arguments(pkg):
    lib = pkg.lib()
    P = pkg.default_params()
    assert lib.tfhe_client_encrypt_bits(ctypes.byref(P), None, 3, None, None) == 1
    bad = pkg.default_params()
    bad.N = 1000
    z = np.zeros(4, np.int32)
    p = z.ctypes.data_as(pkg.I32P)
    assert lib.tfhe_client_gate_keyset(ctypes.byref(bad), p, p, p, p) == 1


def test_no_cpu_fallback_when_library_missing(pkg, tmp_path, monkeypatch):
    """The binding refuses to run without the compiled engine."""
    monkeypatch.setattr(pkg, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(pkg, "_LIB", None)
    with pytest.raises(ImportError):
        pkg.lib()


def test_client_test_vector_and_oracle_lookup_table(pkg, oracle, keys):
    """The host test-vector builder equals the oracle's, and the oracle's
    programmable bootstrap with it evaluates the table on padded messages."""
    P = pkg.default_params()
    OP = pyoracle.default_params()
    p = 8
    f = (5 * np.arange(p) + 2) % p
    table = np.array([pkg.mod_switch_to_torus32(int(v), 2 * p) for v in f], np.int32)
    tv = pkg.test_vector(P.N, table)
    assert (tv == oracle.test_vector(P.N, table)).all()
    assert tv[0] == table[0] and tv[P.N - 1] == -table[0] and tv[P.N // 2] == table[p // 2]
    m = np.arange(p)
    pkg.set_seed([94])
    x = pkg.encrypt_phases(P, [pkg.mod_switch_to_torus32(int(v), 2 * p) for v in m], keys["lwe"])
    out = oracle.bootstrap_tv_batch(OP, keys["bk_fft"], keys["ks"], tv, x)
    ph = pkg.phases(out, keys["lwe"]).astype(np.int64) & 0xFFFFFFFF
    assert (((ph * 2 * p + (1 << 31)) >> 32) % (2 * p) == f[m]).all()
