"""Programmable bootstrap (tfhe_gpu_bootstrap_tv): the gate bootstrap's
constant test vector (tfhe_bootstrap_woKS_FFT.cpp:63-66) replaced by a
lookup table.

* a table on p = 8 padded messages (m encrypted at phase m/16) evaluates
  exactly on every sample, with one shared test vector and with one vector
  per sample, with and without the key switch, in both forms;
* output phases agree with the oracle's programmable bootstrap within the
  bootstrap tolerance;
* the constant test vector mu reproduces tfhe_gpu_tfhe_bootstrap_FFT bit for
  bit (same kernels, the vector read from memory instead of computed).
"""
import numpy as np
import pytest

from helpers import wrap_diff

pytestmark = pytest.mark.gpu
FORMS = ("split_fp32", "fp64")
PHASE_TOL = 2 ** 26
PMSG = 8


def _decode(phases, p):
    """Padded message of Torus32 phases: round(phase * 2p) mod 2p."""
    ph = np.asarray(phases, np.int64) & 0xFFFFFFFF
    return ((ph * 2 * p + (1 << 31)) >> 32) % (2 * p)


def _setup(pkg, oracle, keys, P, count, seed):
    rng = np.random.default_rng(seed)
    m = rng.integers(0, PMSG, count)
    pkg.set_seed([seed])
    x = pkg.encrypt_phases(P, [pkg.mod_switch_to_torus32(int(v), 2 * PMSG) for v in m], keys["lwe"])
    return m, x


@pytest.mark.parametrize("form", FORMS)
def test_lookup_table_shared_vector(pkg, engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    count = 200
    m, x = _setup(pkg, oracle, keys, P, count, 91)
    f = (3 * np.arange(PMSG) + 1) % PMSG
    table = np.array([pkg.mod_switch_to_torus32(int(v), 2 * PMSG) for v in f], np.int32)
    tv = pkg.test_vector(P.N, table)
    assert (tv == oracle.test_vector(P.N, table)).all()
    d_x = torch.from_numpy(x).cuda()
    d_tv = torch.from_numpy(tv).cuda()
    d_out = torch.zeros_like(d_x)
    engine.bootstrap_tv(d_out, d_x, d_tv, count, form, stream=s)
    d_u = torch.zeros((count, P.N + 1), dtype=torch.int32, device="cuda")
    engine.bootstrap_tv(d_u, d_x, d_tv, count, form, keyswitch=False, stream=s)
    torch.cuda.synchronize()
    engine.synchronize()
    out = d_out.cpu().numpy()
    assert (_decode(pkg.phases(out, keys["lwe"]), PMSG) == f[m]).all()
    u = d_u.cpu().numpy()
    assert (_decode(pkg.phases(u, keys["tlwe"]), PMSG) == f[m]).all()
    ref = oracle.bootstrap_tv_batch(P, keys["bk_fft"], keys["ks"], tv, x[:8])
    d = wrap_diff(pkg.phases(out[:8], keys["lwe"]), pkg.phases(ref, keys["lwe"]))
    assert np.abs(d).max() <= PHASE_TOL


def test_lookup_table_per_sample_vectors(pkg, engine, oracle, keys, torch_cuda, P):
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    count = 96
    m, x = _setup(pkg, oracle, keys, P, count, 92)
    # sample c evaluates m -> (m + c) mod 8
    tvs = np.stack([pkg.test_vector(P.N, [pkg.mod_switch_to_torus32((v + c) % PMSG, 2 * PMSG)
                                          for v in range(PMSG)]) for c in range(count)])
    d_x = torch.from_numpy(x).cuda()
    d_out = torch.zeros_like(d_x)
    engine.bootstrap_tv(d_out, d_x, torch.from_numpy(tvs).cuda(), count, "split_fp32", tv_stride=P.N,
                        stream=s)
    torch.cuda.synchronize()
    engine.synchronize()
    got = _decode(pkg.phases(d_out.cpu().numpy(), keys["lwe"]), PMSG)
    assert (got == (m + np.arange(count)) % PMSG).all()
    ref = oracle.bootstrap_tv_batch(P, keys["bk_fft"], keys["ks"], tvs[:6], x[:6])
    d = wrap_diff(pkg.phases(d_out.cpu().numpy()[:6], keys["lwe"]), pkg.phases(ref, keys["lwe"]))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.parametrize("form", FORMS)
def test_constant_vector_is_the_gate_bootstrap(pkg, engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    count = 64
    rng = np.random.default_rng(93)
    x = rng.integers(-2 ** 31, 2 ** 31, (count, P.n + 1)).astype(np.int32)
    d_x = torch.from_numpy(x).cuda()
    mu = 2 ** 29
    d_a = torch.zeros_like(d_x)
    d_b = torch.zeros_like(d_x)
    engine.tfhe_bootstrap_FFT(d_a, d_x, mu, count, form, stream=s)
    engine.bootstrap_tv(d_b, d_x, torch.full((P.N,), mu, dtype=torch.int32, device="cuda"), count, form,
                        stream=s)
    torch.cuda.synchronize()
    engine.synchronize()
    assert torch.equal(d_a, d_b)


def test_bad_arguments(pkg, engine, torch_cuda, P):
    torch = torch_cuda
    d = torch.zeros((2, P.n + 1), dtype=torch.int32, device="cuda")
    with pytest.raises(pkg.TfheError):
        engine.bootstrap_tv(d, d, None, 2, "split_fp32")
    with pytest.raises(pkg.TfheError):
        engine.bootstrap_tv(d, d, d, 2, "split_fp32", tv_stride=7)
    with pytest.raises(pkg.TfheError):
        pkg.test_vector(P.N, [])
