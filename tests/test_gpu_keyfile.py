"""Cloud keys into a context from memory (tfhe_gpu_upload_cloud_key) and
from a key file (tfhe_gpu_upload_cloud_key_file, CLOUD_KEY and SECRET_KEY
records): gates then decrypt to the truth in both forms; a file with other
parameters or a damaged one is refused with a status and leaves the
context's keys usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gates_ok(pkg, eng, keys, torch, P, form, seed):
    rng = np.random.default_rng(seed)
    count = 64
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([seed])
    ca = torch.from_numpy(pkg.encrypt_bits(P, a, keys["lwe"])).cuda()
    cb = torch.from_numpy(pkg.encrypt_bits(P, b, keys["lwe"])).cuda()
    out = torch.zeros_like(ca)
    eng.bootsGate("XOR", out, ca, cb, count, form, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    eng.synchronize()
    return bool((pkg.decrypt_bits(P, out.cpu().numpy(), keys["lwe"]) == (a ^ b)).all())


def test_upload_cloud_key_from_memory(pkg, keys, torch_cuda, P):
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_cloud_key(keys["bk"], keys["ks"])
        for form in ("split_fp32", "fp64"):
            assert _gates_ok(pkg, e, keys, torch_cuda, P, form, 101)
    finally:
        e.close()


def test_upload_cloud_key_files(pkg, keys, torch_cuda, P, tmp_path):
    PP = pkg.default_params()
    cloud = str(tmp_path / "cloud.key")
    secret = str(tmp_path / "secret.key")
    pkg.save_cloud_key(cloud, PP, keys["bk"], keys["ks"])
    pkg.save_secret_key(secret, PP, keys["lwe"], keys["tlwe"], keys["bk"], keys["ks"])
    for path in (cloud, secret):
        e = pkg.Engine(pkg.default_params())
        try:
            e.upload_cloud_key_file(path, forms=("split_fp32",))
            assert _gates_ok(pkg, e, keys, torch_cuda, P, "split_fp32", 102)
        finally:
            e.close()


def test_mismatched_or_damaged_file_refused(pkg, keys, torch_cuda, P, tmp_path):
    PP = pkg.default_params()
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_cloud_key(keys["bk"], keys["ks"], forms=("split_fp32",))
        # a stress-set key file does not fit a default-set context
        SP = pkg.stress_params()
        lwe, tlwe, ks, bk = pkg.gate_keyset(SP, [3])
        other = str(tmp_path / "stress.key")
        pkg.save_cloud_key(other, SP, bk, ks)
        with pytest.raises(pkg.TfheError) as ei:
            e.upload_cloud_key_file(other, forms=("split_fp32",))
        assert ei.value.status == 1
        damaged = tmp_path / "damaged.key"
        pkg.save_cloud_key(str(damaged), PP, keys["bk"], keys["ks"])
        raw = bytearray(damaged.read_bytes())
        raw[len(raw) // 3] ^= 0x10
        damaged.write_bytes(bytes(raw))
        with pytest.raises(pkg.TfheError):
            e.upload_cloud_key_file(str(damaged), forms=("split_fp32",))
        assert _gates_ok(pkg, e, keys, torch_cuda, P, "split_fp32", 103)
    finally:
        e.close()
