"""The allocation-free gate entry point (tfhe_gpu_bootsGates_noalloc).

It exists for callers that cannot allocate device memory inside a call
(fixed memory budgets, latency-critical loops where cudaMalloc/cudaFree would
synchronise the device, frameworks that own all device memory).  It must give
the same ciphertexts as tfhe_gpu_bootsGates -- the same kernels on the same
inputs, so bit-identical, which is inside every tolerance the other tests use
-- on consecutive calls that reuse its shared fixed scratch, and it must
refuse batches beyond its fixed limit.  This file is collected last so that a
run stopping at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _batch(oracle, P, keys, count, seed):
    rng = np.random.default_rng(seed)
    gates = rng.integers(0, 10, count).astype(np.int32)
    oracle.set_seed([seed])
    ca = oracle.encrypt_bits(P, rng.integers(0, 2, count), keys["lwe"])
    cb = oracle.encrypt_bits(P, rng.integers(0, 2, count), keys["lwe"])
    return gates, ca, cb


@pytest.mark.parametrize("form", ["split_fp32", "fp64"])
def test_noalloc_matches_bootsGates_on_consecutive_calls(engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    lib = engine.lib
    stream = torch.cuda.current_stream().cuda_stream
    f = 1 if form == "split_fp32" else 0
    # 512 gates fill the fixed scratch to its last word (default set)
    for call, (count, seed) in enumerate(((300, 71), (97, 72), (512, 73))):
        gates, ca, cb = _batch(oracle, P, keys, count, seed)
        d_g, d_ca, d_cb = _dev(torch, gates), _dev(torch, ca), _dev(torch, cb)
        d_ref = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        d_new = torch.full((count, P.n + 1), -1, dtype=torch.int32, device="cuda")
        st = lib.tfhe_gpu_bootsGates(engine.ctx, d_g.data_ptr(), d_ref.data_ptr(), d_ca.data_ptr(),
                                     d_cb.data_ptr(), count, f, stream)
        assert st == 0, lib.tfhe_gpu_last_error(engine.ctx)
        st = lib.tfhe_gpu_bootsGates_noalloc(engine.ctx, d_g.data_ptr(), d_new.data_ptr(),
                                             d_ca.data_ptr(), d_cb.data_ptr(), count, f, stream)
        assert st == 0, lib.tfhe_gpu_last_error(engine.ctx)
        torch.cuda.synchronize()
        ref, new = d_ref.cpu().numpy(), d_new.cpu().numpy()
        assert (new == ref).all(), "call %d differs from tfhe_gpu_bootsGates" % call
        bits = oracle.decrypt_bits(P, new, keys["lwe"])
        assert bits.shape == (count,)


def test_noalloc_rejects_batches_beyond_its_scratch(engine, torch_cuda, P):
    torch = torch_cuda
    lib = engine.lib
    count = 513  # default set: the fixed scratch holds 512 gates
    d = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    g = torch.zeros(count, dtype=torch.int32, device="cuda")
    st = lib.tfhe_gpu_bootsGates_noalloc(engine.ctx, g.data_ptr(), d.data_ptr(), d.data_ptr(),
                                         d.data_ptr(), count, 1, None)
    assert st == 1  # TFHE_GPU_BAD_PARAM
    msg = lib.tfhe_gpu_last_error(engine.ctx).decode()
    assert "at most 512 gates" in msg
    assert ctypes.sizeof(ctypes.c_int32) == 4
