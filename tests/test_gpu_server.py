"""The continuous-batching gate server (tfhe_gpu_server_*), the request loop
of test_bench/server/cloud.c made multi-client.

* circuits (32-bit ripple-carry adder, 16-bit comparator of cloud.c's
  compare_bit chain, 8-bit multiplexer) decrypt to their plaintext result;
* a circuit's output ciphertexts are bit-identical run alone and run in a
  mix with other clients' circuits (every bootstrap is computed
  independently of its batch neighbours) -- within every stated tolerance;
* admission by device memory: with a pool smaller than the sum of the
  circuits, requests wait and still all complete correctly;
* malformed circuits are refused with a status code.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def circuits(pkg):
    return importlib.import_module("tfhe_gb300.circuits")


def _operands(rng, circuits, kind):
    if kind == "adder":
        gates, ni, outs = circuits.ripple_carry_adder(32)
        a, b = (int(v) for v in rng.integers(0, 2 ** 31, 2))
        bits = [(a >> i) & 1 for i in range(32)] + [(b >> i) & 1 for i in range(32)]
    elif kind == "cmp":
        gates, ni, outs = circuits.comparator(16)
        a, b = (int(v) for v in rng.integers(0, 2 ** 16, 2))
        bits = [(a >> i) & 1 for i in range(16)] + [(b >> i) & 1 for i in range(16)]
    else:
        gates, ni, outs = circuits.multiplexer(8)
        bits = list(rng.integers(0, 2, ni))
    return gates, ni, outs, np.array(bits, np.int32)


def _run(srv, jobs, stagger=0):
    """Submit jobs (gates, ninputs, ct, outs) -- all at once, or one every
    `stagger` ticks while the server runs -- and return their outputs in job
    order."""
    pending = list(jobs)
    rids = []
    if not stagger:
        rids = [srv.submit(*j) for j in pending]
        pending = []
    results = {}
    ticks = idle = 0
    while len(results) < len(jobs):
        if pending and ticks % stagger == 0:
            rids.append(srv.submit(*pending.pop(0)))
        ran = srv.step()
        ticks += 1
        for r in rids:
            if r not in results:
                got = srv.poll(r)
                if got is not None:
                    results[r] = got[0]
        idle = idle + 1 if (ran == 0 and not pending) else 0
        assert idle < 5, "server made no progress"
    return [results[r] for r in rids]


@pytest.mark.parametrize("form", ["split_fp32", "fp64"])
def test_circuits_decrypt(pkg, engine, keys, circuits, form):
    P = pkg.default_params()
    rng = np.random.default_rng(81)
    srv = pkg.Server(engine, pool_slots=4096, max_batch=1024, form=form)
    try:
        jobs, truth = [], []
        pkg.set_seed([81])
        for kind in ("adder", "cmp", "mux"):
            gates, ni, outs, bits = _operands(rng, circuits, kind)
            jobs.append((gates, ni, pkg.encrypt_bits(P, bits, keys["lwe"]), outs))
            truth.append(circuits.evaluate(gates, bits, outs))
        outs = _run(srv, jobs)
        for o, t in zip(outs, truth):
            assert (pkg.decrypt_bits(P, o, keys["lwe"]) == t).all()
    finally:
        srv.close()


def test_same_result_alone_and_in_the_mix(pkg, engine, keys, circuits):
    P = pkg.default_params()
    rng = np.random.default_rng(82)
    pkg.set_seed([82])
    probe = _operands(rng, circuits, "adder")
    probe_job = (probe[0], probe[1], pkg.encrypt_bits(P, probe[3], keys["lwe"]), probe[2])
    others = []
    for i in range(12):
        g, ni, outs, bits = _operands(rng, circuits, ("adder", "cmp", "mux")[i % 3])
        others.append((g, ni, pkg.encrypt_bits(P, bits, keys["lwe"]), outs))
    srv = pkg.Server(engine, pool_slots=8192, max_batch=2048)
    try:
        alone = _run(srv, [probe_job])[0]
        # in the mix: the probe arrives while others are already running
        mixed = _run(srv, others[:6] + [probe_job] + others[6:], stagger=3)[6]
    finally:
        srv.close()
    assert (alone == mixed).all()
    want = circuits.evaluate(probe[0], probe[3], probe[2])
    assert (pkg.decrypt_bits(P, mixed, keys["lwe"]) == want).all()


def test_admission_by_pool_memory(pkg, engine, keys, circuits):
    """Five adders (221 wires each) through a 300-slot pool: one at a time."""
    P = pkg.default_params()
    rng = np.random.default_rng(83)
    pkg.set_seed([83])
    jobs, truth = [], []
    for _ in range(5):
        g, ni, outs, bits = _operands(rng, circuits, "adder")
        jobs.append((g, ni, pkg.encrypt_bits(P, bits, keys["lwe"]), outs))
        truth.append(circuits.evaluate(g, bits, outs))
    srv = pkg.Server(engine, pool_slots=300, max_batch=512)
    try:
        rids = [srv.submit(*j) for j in jobs]
        srv.step()
        st = srv.stats()
        assert st["active"] == 1 and st["queued"] == 4
        results = {}
        while len(results) < 5:
            srv.step()
            for r in rids:
                if r not in results:
                    got = srv.poll(r)
                    if got is not None:
                        results[r] = got[0]
        for r, t in zip(rids, truth):
            assert (pkg.decrypt_bits(P, results[r], keys["lwe"]) == t).all()
        st = srv.stats()
        assert st["free_slots"] == 300 and st["active"] == 0 and st["queued"] == 0
        assert len(st["gate_latency_s"]) == 5 * circuits.bootstraps(jobs[0][0])
    finally:
        srv.close()


def test_bad_circuits_are_refused(pkg, engine, circuits):
    srv = pkg.Server(engine, pool_slots=64, max_batch=16)
    try:
        ct = np.zeros((2, pkg.default_params().n + 1), np.int32)
        with pytest.raises(pkg.TfheError):
            srv.submit([(0, 0, 5, -1)], 2, ct, [2])      # input wire not earlier
        with pytest.raises(pkg.TfheError):
            srv.submit([(42, 0, 1, -1)], 2, ct, [2])     # unknown type
        with pytest.raises(pkg.TfheError):
            srv.submit([(0, 0, 1, -1)], 2, ct, [9])      # bad output wire
        big = np.zeros((100, 4), np.int32)
        with pytest.raises(pkg.TfheError):
            srv.submit(big, 2, ct, [2])                   # more wires than slots
    finally:
        srv.close()


def test_burst_of_circuits_pipelined(pkg, engine, keys, circuits):
    """A burst far above one tick's capacity: 180 circuits submitted at once
    through a server with small batches, so ticks are full, run back to back
    in the pipeline (two in flight) and finish circuits out of submission
    order.  Every request decrypts to its plaintext result, the pool is
    whole again afterwards, and the probe circuit's ciphertexts equal those
    of the same circuit run alone."""
    P = pkg.default_params()
    rng = np.random.default_rng(84)
    pkg.set_seed([84])
    jobs, truth = [], []
    for i in range(180):
        g, ni, outs, bits = _operands(rng, circuits, ("adder", "cmp", "mux")[i % 3])
        jobs.append((g, ni, pkg.encrypt_bits(P, bits, keys["lwe"]), outs))
        truth.append(circuits.evaluate(g, bits, outs))
    srv = pkg.Server(engine, pool_slots=1 << 16, max_batch=600)
    try:
        outs = _run(srv, jobs)
        for o, t in zip(outs, truth):
            assert (pkg.decrypt_bits(P, o, keys["lwe"]) == t).all()
        st = srv.stats()
        assert st["free_slots"] == 1 << 16 and st["active"] == 0
        alone = _run(srv, [jobs[7]])[0]
        assert (alone == outs[7]).all()
    finally:
        srv.close()


def test_long_chain_of_linear_gates(pkg, engine, keys, circuits):
    """200 NOT gates in a chain between two bootstrapped gates: the linear
    gates of a tick run in levels (one launch per level), so a chain longer
    than any small level counter still evaluates in order."""
    P = pkg.default_params()
    B = circuits.Builder(2)
    w = B.gate(circuits.AND, 0, 1)
    for _ in range(200):
        w = B.gate(circuits.NOT, w)
    out = B.gate(circuits.XOR, w, 0)
    gates = B.array()
    pkg.set_seed([85])
    srv = pkg.Server(engine, pool_slots=1024, max_batch=64)
    try:
        for a, b in ((0, 0), (1, 1), (1, 0)):
            ct = pkg.encrypt_bits(P, np.array([a, b], np.int32), keys["lwe"])
            got = _run(srv, [(gates, 2, ct, [out])])[0]
            want = circuits.evaluate(gates, np.array([a, b], np.int32), [out])
            assert (pkg.decrypt_bits(P, got, keys["lwe"]) == want).all()
            assert int(want[0]) == (a & b) ^ a  # 200 NOTs cancel
    finally:
        srv.close()
