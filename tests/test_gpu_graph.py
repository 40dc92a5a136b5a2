"""CUDA graph of a gate batch (tfhe_gpu_graph_*) and the launch-shape
autotuner (tfhe_gpu_autotune).

* a graph replays the same kernels as the eager call on the same buffers:
  outputs bit-identical to the eager ones, twice in a row, decrypting to the
  truth;
* the graph owns its intermediate buffers: a larger eager call on the same
  context in between (which regrows the context's scratch) does not disturb
  it;
* the autotuner returns one of the documented shapes, keeps it, and the
  results under it stay correct.
"""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _inputs(oracle, keys, P, count, seed):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    oracle.set_seed([seed])
    ca = oracle.encrypt_bits(P, a, keys["lwe"])
    cb = oracle.encrypt_bits(P, b, keys["lwe"])
    gates = rng.integers(0, 10, count).astype(np.int32)
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    return gates, ca, cb, truth


def test_graph_matches_eager(pkg, engine, oracle, keys, torch_cuda, P):
    torch = torch_cuda
    s = torch.cuda.current_stream().cuda_stream
    count = 300
    gates, ca, cb, truth = _inputs(oracle, keys, P, count, 71)
    d_g = torch.from_numpy(gates).cuda()
    d_ca = torch.from_numpy(ca).cuda()
    d_cb = torch.from_numpy(cb).cuda()
    for form in ("split_fp32", "fp64"):
        d_eager = torch.zeros_like(d_ca)
        engine.bootsGates(d_g, d_eager, d_ca, d_cb, count, form, stream=s)
        torch.cuda.synchronize()
        d_out = torch.zeros_like(d_ca)
        g = engine.graph_gates(d_g, d_out, d_ca, d_cb, count, form)
        try:
            assert g.kernels >= 3
            for _ in range(2):
                d_out.zero_()
                g.launch(stream=s)
                torch.cuda.synchronize()
                engine.synchronize()
                assert torch.equal(d_out, d_eager)
            # a larger eager batch regrows the context's scratch; the graph
            # keeps its own buffers
            big = 2 * count
            d_big = torch.zeros((big, P.n + 1), dtype=torch.int32, device="cuda")
            engine.bootsGates(torch.cat([d_g, d_g]), d_big, torch.cat([d_ca, d_ca]), torch.cat([d_cb, d_cb]),
                              big, form, stream=s)
            d_out.zero_()
            g.launch(stream=s)
            torch.cuda.synchronize()
            assert torch.equal(d_out, d_eager)
        finally:
            g.close()
        got = d_out.cpu().numpy()
        assert (oracle.decrypt_bits(P, got, keys["lwe"]) == truth).all()


def test_graph_rejects_bad_arguments(pkg, engine, torch_cuda, P):
    torch = torch_cuda
    d = torch.zeros((4, P.n + 1), dtype=torch.int32, device="cuda")
    with pytest.raises(pkg.TfheError) as ei:
        engine.graph_gates(None, d, d, d, 0)
    assert ei.value.status == 1
    with pytest.raises(pkg.TfheError):
        engine.graph_gates(None, d, d, d, 4, uniform_gate=12)


def test_autotune_keeps_a_valid_shape(pkg, oracle, keys, torch_cuda, P):
    torch = torch_cuda
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
        e.upload_keyswitch_key(keys["ks"])
        shape, ms = e.autotune("split_fp32", 500)
        assert shape in (0, 1, 2, 4, 5, 6, 7, 9, 10, 12, 13) and ms > 0
        assert e.get_groups_per_cta("split_fp32") == shape
        count = 500
        gates, ca, cb, truth = _inputs(oracle, keys, P, count, 72)
        d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        e.bootsGates(torch.from_numpy(gates).cuda(), d_out, torch.from_numpy(ca).cuda(),
                     torch.from_numpy(cb).cuda(), count, "split_fp32",
                     stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        e.synchronize()
        assert (oracle.decrypt_bits(P, d_out.cpu().numpy(), keys["lwe"]) == truth).all()
    finally:
        e.close()
