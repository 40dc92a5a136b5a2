"""The engine's key / ciphertext file format (include/tfhe_keyfile.h): round
trips are bit-exact, and malformed files (bad magic, unknown version, wrong
kind, truncation, a flipped payload byte) are refused with a status code and
no output.  CPU only."""
import numpy as np
import pytest


def test_cloud_key_round_trip(pkg, keys, tmp_path):
    P = pkg.default_params()
    path = str(tmp_path / "cloud.key")
    pkg.save_cloud_key(path, P, keys["bk"], keys["ks"])
    P2, bk, ks = pkg.load_cloud_key(path)
    assert (bk == keys["bk"]).all() and (ks == keys["ks"]).all()
    for f in ("n", "N", "k", "l", "Bgbit", "ks_t", "ks_basebit", "lwe_alpha", "tlwe_alpha"):
        assert getattr(P2, f) == getattr(P, f)
    assert [k for k, _ in pkg.keyfile_records(path)] == [pkg.KEYFILE_CLOUD_KEY]


def test_secret_key_round_trip(pkg, keys, tmp_path):
    P = pkg.default_params()
    path = str(tmp_path / "secret.key")
    pkg.save_secret_key(path, P, keys["lwe"], keys["tlwe"], keys["bk"], keys["ks"])
    _, lwe, tlwe, bk, ks = pkg.load_secret_key(path)
    for a, b in ((lwe, keys["lwe"]), (tlwe, keys["tlwe"]), (bk, keys["bk"]), (ks, keys["ks"])):
        assert (a == b).all()


def test_ciphertext_records_append(pkg, keys, tmp_path):
    P = pkg.default_params()
    pkg.set_seed([3])
    c1 = pkg.encrypt_bits(P, [1, 0, 1], keys["lwe"])
    c2 = pkg.encrypt_bits(P, [0, 0, 1, 1, 1], keys["lwe"])
    path = str(tmp_path / "ct.data")
    pkg.save_ciphertexts(path, P, c1)
    pkg.save_ciphertexts(path, P, c2, append=True)
    got = pkg.load_ciphertexts(path)
    assert (got == np.concatenate([c1, c2])).all()
    assert [k for k, _ in pkg.keyfile_records(path)] == [pkg.KEYFILE_CIPHERTEXTS] * 2
    empty = str(tmp_path / "empty.data")
    pkg.save_ciphertexts(empty, P, np.zeros((0, P.n + 1), np.int32))
    assert pkg.load_ciphertexts(empty).shape == (0, P.n + 1)


@pytest.mark.parametrize("damage", ["magic", "version", "kind", "truncate", "payload", "size"])
def test_malformed_files_refused(pkg, keys, tmp_path, damage):
    P = pkg.default_params()
    path = tmp_path / "cloud.key"
    pkg.save_cloud_key(str(path), P, keys["bk"], keys["ks"])
    raw = bytearray(path.read_bytes())
    if damage == "magic":
        raw[0] ^= 0xFF
    elif damage == "version":
        raw[8] = 99
    elif damage == "kind":
        raw[12] = 4  # says ciphertexts
    elif damage == "truncate":
        raw = raw[:len(raw) - 100]
    elif damage == "payload":
        raw[len(raw) // 2] ^= 0x01  # one bit of the key-switching key
    elif damage == "size":
        raw[16] ^= 0x04
    path.write_bytes(bytes(raw))
    with pytest.raises(pkg.TfheError) as ei:
        pkg.load_cloud_key(str(path))
    assert ei.value.status == 1


def test_key_words_match_layout(pkg):
    P = pkg.default_params()
    lib = pkg.lib()
    assert lib.tfhe_keyfile_bk_words(pkg.ctypes.byref(P)) == P.n * P.tgsw_words()
    assert lib.tfhe_keyfile_ks_words(pkg.ctypes.byref(P)) == P.ks_words()
