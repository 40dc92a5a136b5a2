"""Golden fixtures (tests/golden/golden_default.npz, made by
tests/golden/make_golden.py from the pinned oracle) checked against the
oracle on the CPU and against the engine on the GPU."""
import hashlib
import os

import numpy as np
import pytest

from helpers import wrap_diff
from oracle import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_default.npz")
PHASE_TOL = 2 ** 26


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLDEN))


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def test_keys_reproduce(gold, keys, pkg):
    want = list(gold["key_sha"])
    assert [_sha(keys[k]) for k in ("lwe", "tlwe", "ks", "bk")] == want
    P = pkg.default_params()
    assert [_sha(x) for x in pkg.gate_keyset(P, [0])] == want


def test_integer_fixtures(gold, oracle, keys, P):
    assert (oracle.keyswitch(P, keys["ks"], gold["ks_in"]) == gold["ks_out"]).all()
    assert all(oracle.mod_switch_from_torus32(int(v), 2048) == w
               for v, w in zip(gold["ms_in"], gold["ms_out"]))
    assert (oracle.extern_mul_exact(P, gold["ep_acc"], gold["ep_gsw"]) == gold["ep_exact"]).all()
    fft = oracle.extern_mul_fft(P, gold["ep_acc"], oracle.tgsw_to_fft(P, gold["ep_gsw"]))
    assert np.abs(wrap_diff(fft, gold["ep_exact"])).max() <= 2


def test_gate_fixtures_oracle(gold, oracle, keys, P):
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y)
                      for g, x, y in zip(gold["gate_ids"], gold["gate_bits_a"], gold["gate_bits_b"])])
    assert (oracle.decrypt_bits(P, gold["gate_out"], keys["lwe"]) == truth).all()
    out = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], gold["gate_ids"], gold["gate_ca"],
                                  gold["gate_cb"])
    d = wrap_diff(oracle.phases(out, keys["lwe"], P.n), oracle.phases(gold["gate_out"], keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "split_fp32"])
def test_gate_fixtures_engine(gold, engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    count = len(gold["gate_ids"])
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    engine.bootsGates(torch.from_numpy(gold["gate_ids"]).cuda(), d_out,
                      torch.from_numpy(gold["gate_ca"]).cuda(), torch.from_numpy(gold["gate_cb"]).cuda(),
                      count, form, stream=s)
    torch.cuda.synchronize()
    got = d_out.cpu().numpy()
    assert (oracle.decrypt_bits(P, got, keys["lwe"]) == oracle.decrypt_bits(P, gold["gate_out"], keys["lwe"])).all()
    d = wrap_diff(oracle.phases(got, keys["lwe"], P.n), oracle.phases(gold["gate_out"], keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.gpu
def test_integer_fixtures_engine(gold, engine, torch_cuda, P):
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    d_out = torch.zeros((1, P.n + 1), dtype=torch.int32, device="cuda")
    engine.lweKeySwitch(d_out, torch.from_numpy(gold["ks_in"][None]).cuda(), 1, stream=s)
    torch.cuda.synchronize()
    assert (d_out.cpu().numpy()[0] == gold["ks_out"]).all()
    for form, tol in (("fp64", 2), ("split_fp32", 2 ** 16)):
        nb = engine.tgsw_fft_bytes(form)
        d_g = torch.zeros(nb, dtype=torch.uint8, device="cuda")
        engine.tgsw_to_fft(torch.from_numpy(gold["ep_gsw"]).cuda(), d_g, 1, form, stream=s)
        d_acc = torch.from_numpy(gold["ep_acc"][None].copy()).cuda()
        engine.tGswFFTExternMulToTLwe(d_acc, d_g, 1, form, stream=s)
        torch.cuda.synchronize()
        assert np.abs(wrap_diff(d_acc.cpu().numpy()[0], gold["ep_exact"])).max() <= tol
