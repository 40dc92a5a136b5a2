"""GPU parity of the blind rotation, the bootstrap and the gates against the
CPU oracle, through the C ABI.

Criteria: every decrypted gate output equals the oracle's
and the plaintext truth; output phases agree with the oracle's within
2^-6 of a turn (2^26 units).  Phases cannot agree more tightly in general:
one rounding difference between two FFT implementations can move a gadget
digit across its boundary, after which the two accumulators carry different
masks and independent noise terms (bootstrapping noise ~2^-9 of a turn for
the default set).  The decision margin is 1/8 of a turn.
"""
import numpy as np
import pytest

from helpers import tlwe_phase, wrap_diff
from oracle import pyoracle

pytestmark = pytest.mark.gpu

FORMS = ["fp64", "split_fp32"]
PHASE_TOL = 2 ** 26


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def cur(torch):
    return torch.cuda.current_stream().cuda_stream


@pytest.fixture(scope="module")
def inputs(oracle, keys, P):
    rng = np.random.default_rng(1)
    a = rng.integers(0, 2, 64)
    b = rng.integers(0, 2, 64)
    oracle.set_seed([1])
    ca = oracle.encrypt_bits(P, a, keys["lwe"])
    cb = oracle.encrypt_bits(P, b, keys["lwe"])
    return a, b, ca, cb


@pytest.mark.parametrize("form", FORMS)
def test_blind_rotate_vs_oracle(engine, oracle, keys, torch_cuda, P, inputs, form):
    torch = torch_cuda
    _, _, ca, cb = inputs
    count = 3
    xs = np.stack([oracle.gate_combine(P, "NAND", ca[i], cb[i]) for i in range(count)])
    pro = [oracle.bootstrap_prologue(P, 2 ** 29, xs[i]) for i in range(count)]
    bara = np.stack([p[0] for p in pro])
    acc0 = np.stack([p[1] for p in pro])
    d_acc = dev(torch, acc0)
    engine.tfhe_blindRotate_FFT(d_acc, dev(torch, bara), count, form, stream=cur(torch))
    torch.cuda.synchronize()
    got = host(d_acc)
    for i in range(count):
        want = oracle.blind_rotate_fft(P, acc0[i], keys["bk_fft"], bara[i])
        d = wrap_diff(tlwe_phase(got[i], keys["tlwe"], P.N), tlwe_phase(want, keys["tlwe"], P.N))
        assert np.abs(d).max() <= PHASE_TOL, (form, np.abs(d).max())


def test_blind_rotate_zero_steps_is_identity(engine, torch_cuda, P):
    torch = torch_cuda
    rng = np.random.default_rng(2)
    acc = rng.integers(-2 ** 31, 2 ** 31, (2, 2 * P.N)).astype(np.int32)
    bara = np.zeros((2, P.n), np.int32)
    for form in FORMS:
        d_acc = dev(torch, acc)
        engine.tfhe_blindRotate_FFT(d_acc, dev(torch, bara), 2, form, stream=cur(torch))
        torch.cuda.synchronize()
        assert (host(d_acc) == acc).all()


@pytest.mark.parametrize("form", FORMS)
def test_bootstrap_wo_ks_vs_oracle(engine, oracle, keys, torch_cuda, P, inputs, form):
    torch = torch_cuda
    _, _, ca, cb = inputs
    count = 4
    xs = np.stack([oracle.gate_combine(P, "AND", ca[i], cb[i]) for i in range(count)])
    d_out = torch.zeros((count, P.N + 1), dtype=torch.int32, device="cuda")
    mu = 2 ** 29
    engine.tfhe_bootstrap_woKS_FFT(d_out, dev(torch, xs), mu, count, form, stream=cur(torch))
    torch.cuda.synchronize()
    got = host(d_out)
    for i in range(count):
        want = oracle.bootstrap_woks(P, keys["bk_fft"], mu, xs[i])
        pg = oracle.phases(got[i], keys["tlwe"], P.N)[0]
        pw = oracle.phases(want, keys["tlwe"], P.N)[0]
        assert abs(int(wrap_diff(pg, pw))) <= PHASE_TOL
        assert np.sign(pg) == np.sign(pw)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("gate", sorted(pyoracle.GATES))
def test_gate_truth_table(engine, oracle, keys, torch_cuda, P, form, gate):
    torch = torch_cuda
    a = np.array([0, 0, 1, 1])
    b = np.array([0, 1, 0, 1])
    oracle.set_seed([3])
    ca = oracle.encrypt_bits(P, a, keys["lwe"])
    cb = oracle.encrypt_bits(P, b, keys["lwe"])
    d_out = torch.zeros((4, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsGate(gate, d_out, dev(torch, ca), dev(torch, cb), 4, form, stream=cur(torch))
    torch.cuda.synchronize()
    got = oracle.decrypt_bits(P, host(d_out), keys["lwe"])
    want = np.array([pyoracle.GATE_FN[gate](x, y) for x, y in zip(a, b)])
    assert (got == want).all()


@pytest.mark.parametrize("form", FORMS)
def test_mixed_gates_vs_oracle(engine, oracle, keys, torch_cuda, P, inputs, form):
    """A mixed batch: same decrypted bits as the oracle and the truth, phases
    within tolerance of the oracle's."""
    torch = torch_cuda
    a, b, ca, cb = inputs
    count = len(a)
    rng = np.random.default_rng(4)
    gates = rng.integers(0, 10, count).astype(np.int32)
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsGates(dev(torch, gates), d_out, dev(torch, ca), dev(torch, cb), count, form,
                      stream=cur(torch))
    torch.cuda.synchronize()
    got = host(d_out)
    ref = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], gates, ca, cb)
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    assert (oracle.decrypt_bits(P, got, keys["lwe"]) == truth).all()
    assert (oracle.decrypt_bits(P, ref, keys["lwe"]) == truth).all()
    d = wrap_diff(oracle.phases(got, keys["lwe"], P.n), oracle.phases(ref, keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.parametrize("form", FORMS)
def test_known_answer_499_or_388(pkg, oracle, torch_cuda, form):
    """test_bench/ end to end on the GPU, through the host-buffer entry point."""
    P = pkg.default_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [314, 1592, 657])
    c1 = pkg.encrypt_bits(P, [(499 >> i) & 1 for i in range(16)], lwe)
    c2 = pkg.encrypt_bits(P, [(388 >> i) & 1 for i in range(16)], lwe)
    e = pkg.Engine(P)
    try:
        e.upload_bootstrapping_key(bk, forms=(form,))
        e.upload_keyswitch_key(ks)
        out = e.bootsGates_host(c1, c2, gate="OR", form=form)
    finally:
        e.close()
    bits = pkg.decrypt_bits(P, out, lwe)
    assert sum(int(x) << i for i, x in enumerate(bits)) == 503


@pytest.mark.parametrize("form", FORMS)
def test_mux(engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    combos = np.array([(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)])
    oracle.set_seed([5])
    enc = [oracle.encrypt_bits(P, combos[:, i], keys["lwe"]) for i in range(3)]
    d_out = torch.zeros((8, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsMUX(d_out, dev(torch, enc[0]), dev(torch, enc[1]), dev(torch, enc[2]), 8, form,
                    stream=cur(torch))
    torch.cuda.synchronize()
    got = oracle.decrypt_bits(P, host(d_out), keys["lwe"])
    want = np.where(combos[:, 0] == 1, combos[:, 1], combos[:, 2])
    assert (got == want).all()
    ref = np.stack([oracle.boots_mux(P, keys["bk_fft"], keys["ks"], enc[0][i], enc[1][i], enc[2][i])
                    for i in range(2)])
    d = wrap_diff(oracle.phases(host(d_out)[:2], keys["lwe"], P.n), oracle.phases(ref, keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.parametrize("form", FORMS)
def test_large_batch_no_failures(engine, pkg, keys, torch_cuda, P, form):
    """4096 random gates in one call (the batched circuit-layer size): every
    output decrypts to the truth; output noise well inside the margin."""
    torch = torch_cuda
    rng = np.random.default_rng(6)
    count = 4096
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    gates = rng.integers(0, 10, count).astype(np.int32)
    pkg.set_seed([6])
    ca = pkg.encrypt_bits(pkg.default_params(), a, keys["lwe"])
    cb = pkg.encrypt_bits(pkg.default_params(), b, keys["lwe"])
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsGates(dev(torch, gates), d_out, dev(torch, ca), dev(torch, cb), count, form,
                      stream=cur(torch))
    torch.cuda.synchronize()
    out = host(d_out)
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    got = pkg.decrypt_bits(pkg.default_params(), out, keys["lwe"])
    assert (got == truth).all()
    ph = pkg.phases(out, keys["lwe"]).astype(np.int64)
    err = np.abs(np.abs(ph) - 2 ** 29)
    print("%s: output |phase - mu| max 2^%.2f mean 2^%.2f of a turn"
          % (form, np.log2(err.max()) - 32, np.log2(err.mean()) - 32))
    assert err.max() < 2 ** 28  # under 1/16 of a turn


def test_errors_are_status_codes(pkg, keys, torch_cuda, P):
    torch = torch_cuda
    e = pkg.Engine(pkg.default_params())
    try:
        d = torch.zeros((1, P.n + 1), dtype=torch.int32, device="cuda")
        with pytest.raises(pkg.TfheError) as ei:
            e.bootsGate("NAND", d, d, d, 1, "fp64")
        assert ei.value.status == 5  # NO_KEY
        e.upload_bootstrapping_key(keys["bk"], forms=("fp64",))
        with pytest.raises(pkg.TfheError) as ei:
            e.bootsGate("NAND", d, d, d, 1, "fp64")  # KS key missing
        assert ei.value.status == 5
        with pytest.raises(pkg.TfheError) as ei:
            e.bootsGate("NAND", d, d, d, 1, "split_fp32")  # form not built
        assert ei.value.status == 5
        with pytest.raises(pkg.TfheError) as ei:
            e.bootsGate("NAND", d, d, d, 1, 7)
        assert ei.value.status == 1
        e.upload_keyswitch_key(keys["ks"])
        e.bootsGate("NAND", d, d, d, 0, "fp64")  # empty batch is a no-op
        e.synchronize()
    finally:
        e.close()


@pytest.mark.parametrize("form,groups", [("split_fp32", 0), ("split_fp32", 1), ("split_fp32", 2),
                                         ("split_fp32", 4), ("split_fp32", 5), ("split_fp32", 6),
                                         ("split_fp32", 7), ("split_fp32", 8), ("split_fp32", 9),
                                         ("split_fp32", 10), ("split_fp32", 11), ("split_fp32", 12),
                                         ("split_fp32", 13), ("split_fp32", 14),
                                         ("split_fp32", 15), ("split_fp32", 16), ("fp64", 3),
                                         ("fp64", 4), ("fp64", 0), ("fp64", 16)])
def test_every_launch_shape(pkg, oracle, keys, torch_cuda, P, inputs, form, groups):
    """Each blind-rotation launch shape (L2-direct and shared-ring kernels) on
    a ragged batch: decrypted bits equal the truth and the oracle's, phases
    within tolerance, no device timeout."""
    torch = torch_cuda
    a, b, ca, cb = inputs
    count = 37  # not a multiple of any group count: the last CTA is partial
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=(form,))
        e.upload_keyswitch_key(keys["ks"])
        e.set_groups_per_cta(form, groups)
        gates = np.arange(count, dtype=np.int32) % 10
        d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        e.bootsGates(dev(torch, gates), d_out, dev(torch, ca[:count]), dev(torch, cb[:count]), count,
                     form, stream=cur(torch))
        torch.cuda.synchronize()
        e.synchronize()  # raises on a device-side timeout
        got = host(d_out)
    finally:
        e.close()
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a[:count], b[:count])])
    assert (oracle.decrypt_bits(P, got, keys["lwe"]) == truth).all()
    ref = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], gates[:4], ca[:4], cb[:4])
    d = wrap_diff(oracle.phases(got[:4], keys["lwe"], P.n), oracle.phases(ref, keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.parametrize("tail", [40, 200, 400])
def test_auto_shape_full_wave_and_tail(pkg, oracle, keys, torch_cuda, P, inputs, tail):
    """The automatic split-FP32 shape on one full wave (6 per SM on the ring
    kernel with transforms two at a time) plus a tail on the spread kernel
    (40), the pair kernel (200) or the 4-per-SM batched ring kernel (400):
    every output decrypts to the truth and ciphertexts from both launches
    match the oracle's phases."""
    torch = torch_cuda
    a, b, ca, cb = inputs
    count = 6 * 152 + tail
    reps = (count + len(a) - 1) // len(a)
    a, b = np.tile(a, reps)[:count], np.tile(b, reps)[:count]
    ca, cb = np.tile(ca, (reps, 1))[:count], np.tile(cb, (reps, 1))[:count]
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
        e.upload_keyswitch_key(keys["ks"])
        assert e.get_groups_per_cta("split_fp32") == 0
        gates = (np.arange(count, dtype=np.int32) * 7) % 10
        d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        e.bootsGates(dev(torch, gates), d_out, dev(torch, ca), dev(torch, cb), count, "split_fp32",
                     stream=cur(torch))
        torch.cuda.synchronize()
        e.synchronize()
        got = host(d_out)
    finally:
        e.close()
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    assert (oracle.decrypt_bits(P, got, keys["lwe"]) == truth).all()
    idx = np.array([0, 1, 911, 912, 913, count - 1])
    ref = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], gates[idx], ca[idx], cb[idx])
    d = wrap_diff(oracle.phases(got[idx], keys["lwe"], P.n), oracle.phases(ref, keys["lwe"], P.n))
    assert np.abs(d).max() <= PHASE_TOL


@pytest.mark.parametrize("params", ["default", "stress"])
def test_gpu_keyset_is_the_host_keyset(pkg, oracle, torch_cuda, params):
    """tfhe_gpu_gate_keyset (random values on the host, products on the GPU)
    gives the same keys bit for bit as the host keygen from the same seed,
    and the keys it uploaded bootstrap correctly."""
    P = pkg.default_params() if params == "default" else pkg.stress_params()
    want = pkg.gate_keyset(P, [31, 41])
    e = pkg.Engine(P)
    try:
        got = e.gate_keyset([31, 41])
        for a, b in zip(got, want):
            assert (a == b).all()
        torch = torch_cuda
        rng = np.random.default_rng(95)
        bits = rng.integers(0, 2, (2, 16))
        pkg.set_seed([95])
        ca = pkg.encrypt_bits(P, bits[0], got[0])
        cb = pkg.encrypt_bits(P, bits[1], got[0])
        d_out = torch.zeros((16, P.n + 1), dtype=torch.int32, device="cuda")
        for form in ("split_fp32", "fp64"):
            e.bootsGate("NAND", d_out, torch.from_numpy(ca).cuda(), torch.from_numpy(cb).cuda(), 16, form,
                        stream=torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            e.synchronize()
            assert (pkg.decrypt_bits(P, d_out.cpu().numpy(), got[0]) == 1 - (bits[0] & bits[1])).all()
    finally:
        e.close()


def test_stress_set_noise_band(pkg, torch_cuda):
    """The alternative set (n=500, l=2, Bgbit=10, TRLWE 2^-24) is noisy by
    design: its bootstrapping noise n (k+1) l N Var(digit) alpha^2 =
    500 * 4 * 1024 * (2^18 / 3) * 2^-48 ~ 2^-10.6 (sigma ~ 0.025 turn) puts the
    1/8-turn decision margin at ~4.3 sigma, i.e. about one failure per 10^5
    gates in any exact implementation.  Both forms must show that noise and
    no more: sigma of the output phase error in [0.02, 0.035] turn, the two
    forms within 10 % of each other (the automatic split point s = 26 gives
    about 4 %; s = 27 gave 15 %), at most 4 failures in 16384 gates."""
    torch = torch_cuda
    P = pkg.stress_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    e = pkg.Engine(P)
    try:
        e.upload_bootstrapping_key(bk)
        e.upload_keyswitch_key(ks)
        total = 16384
        rng = np.random.default_rng(96)
        a = rng.integers(0, 2, total)
        b = rng.integers(0, 2, total)
        pkg.set_seed([96])
        d_a = torch.from_numpy(pkg.encrypt_bits(P, a, lwe)).cuda()
        d_b = torch.from_numpy(pkg.encrypt_bits(P, b, lwe)).cuda()
        sig = {}
        for form in ("split_fp32", "fp64"):
            d_out = torch.empty_like(d_a)
            e.bootsGate("NAND", d_out, d_a, d_b, total, form, stream=torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            e.synchronize()
            out = d_out.cpu().numpy()
            fails = int((pkg.decrypt_bits(P, out, lwe) != 1 - (a & b)).sum())
            ph = pkg.phases(out, lwe).astype(np.int64)
            want = np.where(1 - (a & b) == 1, 2 ** 29, -(2 ** 29))
            err = ((ph - want + 2 ** 31) % 2 ** 32 - 2 ** 31) / 2.0 ** 32
            sig[form] = float(err.std())
            assert 0.02 <= sig[form] <= 0.035, (form, sig[form])
            assert fails <= 4, (form, fails)
        assert abs(sig["split_fp32"] / sig["fp64"] - 1) <= 0.10, sig
        assert e.params.split_bits == 26
    finally:
        e.close()


@pytest.mark.parametrize("groups,count", [(11, 8), (6, 6), (9, 9), (10, 7), (13, 5), (5, 5)])
def test_bounded_waits_report_timeout(pkg, oracle, keys, torch_cuda, P, inputs, groups, count):
    """The device-side failure path without a fault: a blind rotation whose
    key-row stream never starts (a flag the producer honours) makes every
    consumer's bounded wait run out; the kernel ends within a few seconds,
    the host gets TFHE_GPU_TIMEOUT, and the same context then bootstraps
    correctly.  Shapes: pair (1 and 3 per CTA), ring in line, the two
    batched rings, ring with a producer warp."""
    import time
    torch = torch_cuda
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
        e.upload_keyswitch_key(keys["ks"])
        e.set_groups_per_cta("split_fp32", groups)
        t0 = time.perf_counter()
        st = e.selftest_timeout("split_fp32", count)
        took = time.perf_counter() - t0
        assert st == 3, st
        assert took < 30, took
        e.synchronize()  # status word cleared: no stale timeout
        a, b, ca, cb = inputs
        d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        e.bootsGate("AND", d_out, dev(torch, ca[:count]), dev(torch, cb[:count]), count, "split_fp32",
                    stream=cur(torch))
        torch.cuda.synchronize()
        e.synchronize()
        assert (oracle.decrypt_bits(P, host(d_out), keys["lwe"]) == (a[:count] & b[:count])).all()
    finally:
        e.close()


def test_l2_shapes_have_no_waits(pkg, keys, torch_cuda):
    """Shapes that read key rows straight from L2 (FP64 shape 3, and the
    split-FP32 spread kernel that small batches take automatically) have no
    key ring to stall: the self-test finds no timeout."""
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("fp64", "split_fp32"))
        e.set_groups_per_cta("fp64", 3)
        assert e.selftest_timeout("fp64", 3) == 0
        assert e.get_groups_per_cta("split_fp32") == 0
        assert e.selftest_timeout("split_fp32", 8) == 0
    finally:
        e.close()


@pytest.mark.parametrize("count", [76, 77, 152, 153, 304, 305, 608, 609, 912, 913, 988, 989, 1064, 1065, 1216,
                                   1217, 1520, 1521])
def test_auto_shape_boundaries(pkg, engine, oracle, keys, torch_cuda, P, count):
    """Batch sizes on both sides of the automatic shape's boundaries: the
    cluster spread kernel up to one per two SMs, the spread kernel up to 1
    per SM, the pair kernel up to 2 per SM; one
    4-per-SM wave up to 4 per SM; 6-per-SM waves; a wave plus a spread tail,
    a pair tail, a 4-per-SM tail, or a partial 6-per-SM wave: every output
    decrypts to the truth."""
    torch = torch_cuda
    rng = np.random.default_rng(97 + count)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([97 + count])
    ca = pkg.encrypt_bits(P, a, keys["lwe"])
    cb = pkg.encrypt_bits(P, b, keys["lwe"])
    gates = rng.integers(0, 10, count).astype(np.int32)
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsGates(dev(torch, gates), d_out, dev(torch, ca), dev(torch, cb), count, "split_fp32",
                      stream=cur(torch))
    torch.cuda.synchronize()
    engine.synchronize()
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    assert (pkg.decrypt_bits(P, host(d_out), keys["lwe"]) == truth).all()


@pytest.mark.parametrize("count", [1, 4096])
def test_automatic_shape_is_deterministic(pkg, engine, keys, torch_cuda, P, count):
    """The same batch twice gives bit-identical ciphertexts: a single gate on
    the spread kernel (products summed in a fixed order, integer
    atomics into the accumulator) and a 4096-gate layer whose first key
    switch runs on the side stream during the remainder wave."""
    torch = torch_cuda
    rng = np.random.default_rng(201 + count)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([201 + count])
    d_ca = dev(torch, pkg.encrypt_bits(P, a, keys["lwe"]))
    d_cb = dev(torch, pkg.encrypt_bits(P, b, keys["lwe"]))
    gates = dev(torch, rng.integers(0, 10, count).astype(np.int32))
    outs = []
    for _ in range(2):
        d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
        engine.bootsGates(gates, d_out, d_ca, d_cb, count, "split_fp32", stream=cur(torch))
        torch.cuda.synchronize()
        engine.synchronize()
        outs.append(host(d_out))
    assert (outs[0] == outs[1]).all()


@pytest.mark.parametrize("count", [912 + 100, 912 + 400])
def test_stress_set_split_batches(pkg, torch_cuda, count):
    """The alternative set (l = 2) through the split automatic shape: a
    6-per-SM wave plus a spread-kernel tail (1012), or plus a 4-per-SM tail
    with the first key switch on the side stream (1312).  Every gate
    decrypts to the truth except at the set's own failure rate (about 1e-5
    per gate): at most one failure."""
    torch = torch_cuda
    P = pkg.stress_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    e = pkg.Engine(P)
    try:
        e.upload_bootstrapping_key(bk, forms=("split_fp32",))
        e.upload_keyswitch_key(ks)
        rng = np.random.default_rng(211 + count)
        a = rng.integers(0, 2, count)
        b = rng.integers(0, 2, count)
        pkg.set_seed([211 + count])
        d_a = torch.from_numpy(pkg.encrypt_bits(P, a, lwe)).cuda()
        d_b = torch.from_numpy(pkg.encrypt_bits(P, b, lwe)).cuda()
        d_out = torch.empty_like(d_a)
        e.bootsGate("AND", d_out, d_a, d_b, count, "split_fp32", stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        e.synchronize()
        fails = int((pkg.decrypt_bits(P, d_out.cpu().numpy(), lwe) != (a & b)).sum())
        assert fails <= 1, fails
    finally:
        e.close()


def test_shapes_agree_bit_for_bit(pkg, keys, torch_cuda, P, inputs):
    """Every split-FP32 shape that sums the 2l key rows in order (L2-direct
    1/2/4, the rings 5-10, the spread kernel 14 and its two-SM cluster form
    16, the fixed-order automatic shape 15) runs the same transforms and
    products in the same order, so their ciphertexts are identical bit for
    bit.  The pair kernel adds the two halves' partial products and may
    differ in the last rounding; it is held to the phase tolerance in the
    other tests."""
    torch = torch_cuda
    a, b, ca, cb = inputs
    count = 37
    gates = dev(torch, (np.arange(count, dtype=np.int32) * 3) % 10)
    e = pkg.Engine(pkg.default_params())
    outs = {}
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
        e.upload_keyswitch_key(keys["ks"])
        for shape in (1, 2, 4, 5, 6, 7, 8, 9, 10, 14, 15, 16):
            e.set_groups_per_cta("split_fp32", shape)
            d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
            e.bootsGates(gates, d_out, dev(torch, ca[:count]), dev(torch, cb[:count]), count, "split_fp32",
                         stream=cur(torch))
            torch.cuda.synchronize()
            e.synchronize()
            outs[shape] = host(d_out)
    finally:
        e.close()
    for shape, out in outs.items():
        assert (out == outs[6]).all(), shape


def test_fp32_peak_probe(pkg, torch_cuda):
    """The FP32 FMA-pipe probe behind the roofline denominator: GB300 has
    152 SMs x 128 FP32 lanes at up to 2.07 GHz, 80.5 TFLOP/s nominal."""
    tf, ms = pkg.measure_fp32_peak(0)
    print("measured FP32 FMA peak: %.1f TFLOP/s (%.2f ms)" % (tf, ms))
    assert 40.0 <= tf <= 90.0, tf


def test_fp64_peak_probe(pkg, torch_cuda):
    """The FP64 FMA-pipe probe: GB300's FP64 rate is about 1/64 of FP32."""
    tf, ms = pkg.measure_fp64_peak(0)
    print("measured FP64 FMA peak: %.2f TFLOP/s (%.2f ms)" % (tf, ms))
    assert 0.3 <= tf <= 5.0, tf


@pytest.mark.parametrize("count", [200, 912 + 200])
def test_fixed_order_shape_independent_of_batch(pkg, keys, torch_cuda, P, count):
    """Shape 15 (automatic, fixed summation order) gives every ciphertext the
    same result bit for bit in a batch of `count` (a 2-per-SM remainder,
    which shape 0 runs on the pair kernel) and in a batch of 37 (spread
    kernel)."""
    torch = torch_cuda
    rng = np.random.default_rng(231 + count)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([231 + count])
    ca = pkg.encrypt_bits(P, a, keys["lwe"])
    cb = pkg.encrypt_bits(P, b, keys["lwe"])
    gates = (np.arange(count, dtype=np.int32) * 3) % 10
    e = pkg.Engine(pkg.default_params())
    try:
        e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
        e.upload_keyswitch_key(keys["ks"])
        e.set_groups_per_cta("split_fp32", 15)
        outs = []
        for lo, hi in ((0, count), (count - 37, count)):
            d_out = torch.zeros((hi - lo, P.n + 1), dtype=torch.int32, device="cuda")
            e.bootsGates(dev(torch, gates[lo:hi]), d_out, dev(torch, ca[lo:hi]), dev(torch, cb[lo:hi]), hi - lo,
                         "split_fp32", stream=cur(torch))
            torch.cuda.synchronize()
            e.synchronize()
            outs.append(host(d_out))
    finally:
        e.close()
    assert (outs[0][count - 37:] == outs[1]).all()
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
    assert (pkg.decrypt_bits(P, outs[0], keys["lwe"]) == truth).all()


def test_cluster_spread_kernel_stress_set_bit_for_bit(pkg, torch_cuda):
    """The two-SM cluster kernel (shape 16) on the l = 2 set gives the spread
    kernel's (shape 14) ciphertexts bit for bit, and decrypts to the truth."""
    torch = torch_cuda
    P = pkg.stress_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [0])
    count = 37
    rng = np.random.default_rng(241)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([241])
    d_a = torch.from_numpy(pkg.encrypt_bits(P, a, lwe)).cuda()
    d_b = torch.from_numpy(pkg.encrypt_bits(P, b, lwe)).cuda()
    e = pkg.Engine(P)
    outs = {}
    try:
        e.upload_bootstrapping_key(bk, forms=("split_fp32",))
        e.upload_keyswitch_key(ks)
        for shape in (14, 16):
            e.set_groups_per_cta("split_fp32", shape)
            d_out = torch.empty_like(d_a)
            e.bootsGate("NAND", d_out, d_a, d_b, count, "split_fp32", stream=cur(torch))
            torch.cuda.synchronize()
            e.synchronize()
            outs[shape] = host(d_out)
    finally:
        e.close()
    assert (outs[14] == outs[16]).all()
    assert int((pkg.decrypt_bits(P, outs[16], lwe) != 1 - (a & b)).sum()) <= 1


@pytest.mark.parametrize("params,count", [("default", 21), ("stress", 21), ("default", 150)])
def test_fp64_cluster_kernel_matches_the_other_fp64_shapes(pkg, torch_cuda, params, count):
    """The FP64 two-SM cluster kernel (shape 16, and the automatic shape for
    small batches) runs the same transforms and sums the key rows in the same
    order as the L2-direct FP64 kernel (shape 3): the ciphertexts agree bit
    for bit, and decrypt to the truth (150 gates: two waves of clusters)."""
    torch = torch_cuda
    P = pkg.default_params() if params == "default" else pkg.stress_params()
    lwe, tlwe, ks, bk = pkg.gate_keyset(P, [5])
    rng = np.random.default_rng(251)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    pkg.set_seed([251])
    d_a = torch.from_numpy(pkg.encrypt_bits(P, a, lwe)).cuda()
    d_b = torch.from_numpy(pkg.encrypt_bits(P, b, lwe)).cuda()
    e = pkg.Engine(P)
    outs = {}
    try:
        e.upload_bootstrapping_key(bk, forms=("fp64",))
        e.upload_keyswitch_key(ks)
        assert e.get_groups_per_cta("fp64") == 0
        for shape in (3, 16, 0):
            e.set_groups_per_cta("fp64", shape)
            d_out = torch.empty_like(d_a)
            e.bootsGate("NAND", d_out, d_a, d_b, count, "fp64", stream=cur(torch))
            torch.cuda.synchronize()
            e.synchronize()
            outs[shape] = host(d_out)
    finally:
        e.close()
    assert (outs[3] == outs[16]).all()
    assert (outs[0] == outs[16]).all()
    assert int((pkg.decrypt_bits(P, outs[16], lwe) != 1 - (a & b)).sum()) <= (0 if params == "default" else 1)


@pytest.mark.parametrize("count", [1000, 1])
def test_layer_split_over_contexts(pkg, keys, torch_cuda, P, count):
    """tfhe_gpu_bootsGates_host_split with two contexts (both on GPU 0 here,
    one per GPU in use): the shards run concurrently and the outputs come
    back in layer order, bit-identical to the whole layer on one context
    (fixed summation order, shape 15); a 1-gate layer leaves one context an
    empty shard; the same context twice is refused."""
    rng = np.random.default_rng(251)
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    gates = rng.integers(0, 10, count).astype(np.int32)
    pkg.set_seed([251])
    ca = pkg.encrypt_bits(P, a, keys["lwe"])
    cb = pkg.encrypt_bits(P, b, keys["lwe"])
    engines = [pkg.Engine(pkg.default_params()) for _ in range(3)]
    try:
        for e in engines:
            e.upload_bootstrapping_key(keys["bk"], forms=("split_fp32",))
            e.upload_keyswitch_key(keys["ks"])
            e.set_groups_per_cta("split_fp32", 15)
        whole = engines[0].bootsGates_host(ca, cb, gates=gates)
        split = pkg.bootsGates_host_split(engines[1:], ca, cb, gates=gates)
        assert (split == whole).all()
        names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
        truth = np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])
        assert (pkg.decrypt_bits(P, split, keys["lwe"]) == truth).all()
        with pytest.raises(pkg.TfheError):
            pkg.bootsGates_host_split([engines[1], engines[1]], ca, cb, gates=gates)
    finally:
        for e in engines:
            e.close()
