"""GPU parity against the oracle at the benchmarked sizes, through the C ABI.

What can be compared, and how tightly:

* Integer work is bit-exact (other test files).  The external product is
  compared word by word with the exact int64 negacyclic product, here on all
  1,024 products of the external-product workload: FP64 within 2 units of
  2^-32, split-FP32 within 2^16 units (rms ~2^11).
* A whole bootstrap under a real key cannot agree with another FFT
  implementation to the rounding level: a one-unit rounding difference
  carries some gadget digit across its boundary within the first steps, the
  two accumulators then add different key rows (fresh masks), and from there
  on their noise terms are independent.  The oracle's own FFT bootstrap
  differs from its exact int64 bootstrap in the same way.  So under a real
  key the parity criteria are: identical decrypted bits, and output noise of
  the same distribution as the oracle's (sigma ratio, mean, tail), with the
  phase differences reported as a distribution.
* Under a noiseless trivial key (TGSW(s_i) = s_i * H, no mask, no noise) no
  mask ever becomes random, so nothing amplifies a rounding difference: the
  whole pipeline -- gate combination, modulus switch, test vector, every
  rotation, decomposition, products, extraction, key switch -- must then
  follow the exact int64 oracle word by word on every ciphertext, up to
  additive jumps of the lowest gadget unit.  The decomposition truncates
  below 2^(32 - l Bgbit) (its offset centres the digits, it does not round),
  and this key keeps coefficients exactly on multiples of that unit, so a
  one-unit rounding difference of either sign can move a lowest-level digit
  by one, which moves the result by 2^(32 - l Bgbit) = 2^11 units (default
  set).  Such jumps add up, they do not multiply: the oracle's own FFT
  bootstrap lands up to 2^15.8 (default) / 2^16.8 (stress) units from its
  exact one this way.  The bound is 2^20 units (2^-12 turn), 2^17 below the
  decision margin; any error of structure (a wrong rotation, step, index or
  extraction) moves a result by ~2^29.

Every figure is printed (pytest -s shows them).
"""
import numpy as np
import pytest

from helpers import wrap_diff
from oracle import pyoracle

pytestmark = pytest.mark.gpu

FORMS = ["split_fp32", "fp64"]
GATE_SET = (0, 1, 3, 2)  # NAND, AND, XOR, OR: the batched-layer workload's mix
TURN = 2.0 ** 32


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def cur(torch):
    return torch.cuda.current_stream().cuda_stream


def log2_turn(x):
    return float(np.log2(max(float(x), 1.0)) - 32)


def describe(name, d):
    """One line of |d| statistics, d in units of 2^-32 turn."""
    a = np.abs(np.asarray(d, np.float64))
    return ("%s: |d| p50 2^%.2f p99 2^%.2f max 2^%.2f turn; below 2^-20: %d of %d; below 2^-12: %d"
            % (name, log2_turn(np.percentile(a, 50)), log2_turn(np.percentile(a, 99)), log2_turn(a.max()),
               int((a < 2 ** 12).sum()), len(a), int((a < 2 ** 20).sum())))


def gate_truth(gates, a, b):
    names = sorted(pyoracle.GATES, key=lambda g: pyoracle.GATES[g])
    return np.array([pyoracle.GATE_FN[names[g]](x, y) for g, x, y in zip(gates, a, b)])


def output_noise(phases, bits):
    """Signed phase error against the ideal +-1/8 of the decrypted value."""
    ideal = np.where(np.asarray(bits) == 1, 2 ** 29, -(2 ** 29))
    return wrap_diff(phases, ideal).astype(np.float64)


def trivial_bootstrapping_key(P, lwe_key):
    """Noiseless, maskless TGSW(s_i) = s_i * H: row (poly j, level p) holds
    s_i * 2^(32 - (p+1) Bgbit) at coefficient 0 of polynomial j."""
    bk = np.zeros((P.n, P.kpl, P.k + 1, P.N), np.uint32)
    for j in range(P.k + 1):
        for p in range(P.l):
            h = np.uint32(1 << (32 - (p + 1) * P.Bgbit))
            bk[:, j * P.l + p, j, 0] = lwe_key.astype(np.uint32) * h
    return bk.view(np.int32).reshape(-1)


def run_gates(torch, eng, gates, ca, cb, form):
    d_out = torch.zeros(ca.shape, dtype=torch.int32, device="cuda")
    eng.bootsGates(dev(torch, gates), d_out, dev(torch, ca), dev(torch, cb), len(gates), form,
                   stream=cur(torch))
    torch.cuda.synchronize()
    eng.synchronize()
    return d_out.cpu().numpy()


# ---------------------------------------------------------------------------
# the batched circuit layer: 4,096 mixed gates, default set, both forms
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def layer(oracle, keys, P):
    rng = np.random.default_rng(4)
    count = 4096
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    gates = np.array(GATE_SET, np.int32)[rng.integers(0, len(GATE_SET), count)]
    oracle.set_seed([4])
    ca = oracle.encrypt_bits(P, a, keys["lwe"])
    cb = oracle.encrypt_bits(P, b, keys["lwe"])
    # the reference path (FP64 2N-point transform) on every host thread
    ref = oracle.boots_gate_batch(P, keys["bk_fft"], keys["ks"], gates, ca, cb)
    return {"a": a, "b": b, "gates": gates, "ca": ca, "cb": cb, "ref": ref,
            "truth": gate_truth(gates, a, b)}


@pytest.mark.parametrize("form", FORMS)
def test_layer_4096_against_oracle(engine, oracle, keys, torch_cuda, P, layer, form):
    """All 4,096 gates of the layer: decrypted bits identical to the oracle's
    and to the truth; output noise distributed like the oracle's."""
    got = run_gates(torch_cuda, engine, layer["gates"], layer["ca"], layer["cb"], form)
    bits = oracle.decrypt_bits(P, got, keys["lwe"])
    ref_bits = oracle.decrypt_bits(P, layer["ref"], keys["lwe"])
    assert (ref_bits == layer["truth"]).all()
    assert (bits == layer["truth"]).all(), int((bits != layer["truth"]).sum())
    ph = oracle.phases(got, keys["lwe"], P.n)
    ph_ref = oracle.phases(layer["ref"], keys["lwe"], P.n)
    d = wrap_diff(ph, ph_ref).astype(np.float64)
    e_gpu = output_noise(ph, bits)
    e_ref = output_noise(ph_ref, ref_bits)
    s_gpu, s_ref, s_d = e_gpu.std(), e_ref.std(), d.std()
    print("\n[layer 4096, %s] " % form + describe("engine - oracle", d))
    print("[layer 4096, %s] output noise sigma: engine 2^%.3f, oracle 2^%.3f turn (ratio %.4f); "
          "max |noise| engine 2^%.2f, oracle 2^%.2f; sigma(d) / sqrt(s_e^2 + s_o^2) = %.3f; mean(d) %.2e turn"
          % (form, log2_turn(s_gpu), log2_turn(s_ref), s_gpu / s_ref, log2_turn(np.abs(e_gpu).max()),
             log2_turn(np.abs(e_ref).max()), s_d / np.hypot(s_gpu, s_ref), d.mean() / TURN))
    # the engine's noise is the oracle's noise: same sigma within sampling
    # error (4,096 samples: 1.1 % per sigma), no bias, no heavier tail
    assert 0.9 <= s_gpu / s_ref <= 1.1, (s_gpu, s_ref)
    assert abs(d.mean()) <= 5 * s_d / np.sqrt(len(d))
    assert s_d <= 1.1 * np.hypot(s_gpu, s_ref)
    assert np.abs(e_gpu).max() <= 1.25 * max(np.abs(e_ref).max(), 6 * s_ref)
    assert np.abs(d).max() < 2 ** 28  # 1/16 turn: half the decision margin


TRIVIAL_TOL = 2 ** 20  # units of 2^-32 turn; see the module docstring


@pytest.fixture(scope="module")
def trivial_layer(oracle, keys, P, layer):
    """The layer's gates under the trivial key: the exact int64 oracle on all
    4,096, and the oracle's own FFT bootstrap on the first 256."""
    bk0 = trivial_bootstrapping_key(P, keys["lwe"])
    exact = oracle.boots_gate_exact_batch(P, bk0, keys["ks"], layer["gates"], layer["ca"], layer["cb"])
    m = 256
    fft = oracle.boots_gate_batch(P, oracle.bk_to_fft(P, bk0), keys["ks"], layer["gates"][:m],
                                  layer["ca"][:m], layer["cb"][:m])
    return {"bk0": bk0, "exact": exact, "fft_dev": np.abs(wrap_diff(fft, exact[:m])).max()}


@pytest.mark.parametrize("form", FORMS)
def test_layer_4096_trivial_key_follows_exact_oracle(pkg, oracle, keys, torch_cuda, P, layer, trivial_layer,
                                                     form):
    """The same 4,096 gates under the noiseless trivial bootstrapping key (the
    real key-switching key): every output word follows the exact int64
    oracle's."""
    torch = torch_cuda
    eng = pkg.Engine(pkg.default_params())
    try:
        eng.upload_bootstrapping_key(trivial_layer["bk0"], forms=(form,))
        eng.upload_keyswitch_key(keys["ks"])
        got = run_gates(torch, eng, layer["gates"], layer["ca"], layer["cb"], form)
    finally:
        eng.close()
    d = wrap_diff(got, trivial_layer["exact"])
    print("\n[trivial key, layer 4096, %s] engine - exact: max %d units (2^%.2f), bodies differing %d of %d; "
          "oracle FFT - exact (256 gates): max %d units"
          % (form, np.abs(d).max(), np.log2(np.abs(d).max() + 1), int((d[:, P.n] != 0).sum()), len(d),
             trivial_layer["fft_dev"]))
    # the key switch of the all-zero extracted mask: identical mask words
    assert (d[:, :P.n] == 0).all()
    assert np.abs(d).max() <= TRIVIAL_TOL
    assert (oracle.decrypt_bits(P, got, keys["lwe"]) == layer["truth"]).all()


@pytest.mark.parametrize("form", FORMS)
def test_lookup_table_trivial_key_all_digit_levels(pkg, oracle, keys, torch_cuda, P, form):
    """Programmable bootstrap with a random test vector under the trivial
    key: every gadget level carries non-zero digits in every step, and the
    result must still follow the exact int64 oracle word by word."""
    torch = torch_cuda
    rng = np.random.default_rng(301)
    count = 512
    tv = rng.integers(-2 ** 31, 2 ** 31, P.N).astype(np.int32)
    oracle.set_seed([301])
    x = oracle.encrypt_bits(P, rng.integers(0, 2, count), keys["lwe"])
    x[:, P.n] = rng.integers(-2 ** 31, 2 ** 31, count).astype(np.int32)  # any rotation
    bk0 = trivial_bootstrapping_key(P, keys["lwe"])
    eng = pkg.Engine(pkg.default_params())
    try:
        eng.upload_bootstrapping_key(bk0, forms=(form,))
        eng.upload_keyswitch_key(keys["ks"])
        d_out = torch.zeros((count, P.k * P.N + 1), dtype=torch.int32, device="cuda")
        eng.bootstrap_tv(d_out, dev(torch, x), dev(torch, tv), count, form, keyswitch=False,
                         stream=cur(torch))
        torch.cuda.synchronize()
        eng.synchronize()
        got = d_out.cpu().numpy()
    finally:
        eng.close()
    # the oracle's bootstrap without key switch on this test vector: the
    # same prologue (modulus switch, X^{2N - barb} tv) then the exact
    # blind rotation; with a maskless key the extracted sample is (0, b)
    exact = np.zeros_like(got)
    bara_all = np.zeros((count, P.n), np.int32)
    for c in range(count):
        bara, acc = oracle.bootstrap_prologue(P, 0, x[c])
        barb = oracle.mod_switch_from_torus32(int(x[c, P.n]), 2 * P.N)
        acc[P.k * P.N:] = oracle.mul_by_xai(P.N, (2 * P.N - barb) % (2 * P.N), tv)
        bara_all[c] = bara
        exact[c] = oracle.extract(P, oracle.blind_rotate_exact(P, acc, bk0, bara))
    d = wrap_diff(got, exact)
    print("\n[trivial key, lookup table 512, %s] engine - exact: max %d units, rms %.2f, words differing %d"
          % (form, np.abs(d).max(), float(np.sqrt((d.astype(np.float64) ** 2).mean())), int((d != 0).sum())))
    assert (d[:, :P.k * P.N] == 0).all()
    assert np.abs(d).max() <= TRIVIAL_TOL


# ---------------------------------------------------------------------------
# the alternative (stress) set: n = 500, l = 2, Bgbit = 10
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def stress(pkg, oracle):
    P = pyoracle.stress_params()
    lwe, tlwe, ks, bk = oracle.gate_keyset(P, [0])
    bk_fft = oracle.bk_to_fft(P, bk)
    rng = np.random.default_rng(302)
    count = 1024
    a = rng.integers(0, 2, count)
    b = rng.integers(0, 2, count)
    oracle.set_seed([302])
    ca = oracle.encrypt_bits(P, a, lwe)
    cb = oracle.encrypt_bits(P, b, lwe)
    gates = np.zeros(count, np.int32)  # NAND
    ref = oracle.boots_gate_batch(P, bk_fft, ks, gates, ca, cb)
    return {"P": P, "lwe": lwe, "ks": ks, "bk": bk, "bk_fft": bk_fft, "a": a, "b": b, "ca": ca,
            "cb": cb, "gates": gates, "ref": ref, "truth": 1 - (a & b)}


@pytest.fixture(scope="module")
def stress_engine(pkg, stress, torch_cuda):
    eng = pkg.Engine(pkg.stress_params())
    eng.upload_bootstrapping_key(stress["bk"])
    eng.upload_keyswitch_key(stress["ks"])
    yield eng
    eng.close()


@pytest.mark.parametrize("form", FORMS)
def test_stress_set_1024_nand_against_oracle(stress_engine, oracle, torch_cuda, stress, form):
    """1,024 NAND gates on the stress set: bits identical to the oracle's
    and the truth (the set's own failure rate is ~1e-5 per gate), output
    noise distributed like the oracle's."""
    S = stress
    P = S["P"]
    got = run_gates(torch_cuda, stress_engine, S["gates"], S["ca"], S["cb"], form)
    bits = oracle.decrypt_bits(P, got, S["lwe"])
    ref_bits = oracle.decrypt_bits(P, S["ref"], S["lwe"])
    assert int((bits != S["truth"]).sum()) <= 1
    assert int((ref_bits != S["truth"]).sum()) <= 1
    assert int((bits != ref_bits).sum()) <= 1
    ph = oracle.phases(got, S["lwe"], P.n)
    ph_ref = oracle.phases(S["ref"], S["lwe"], P.n)
    d = wrap_diff(ph, ph_ref).astype(np.float64)
    e_gpu = output_noise(ph, S["truth"])
    e_ref = output_noise(ph_ref, S["truth"])
    s_gpu, s_ref = e_gpu.std(), e_ref.std()
    print("\n[stress 1024 NAND, %s] " % form + describe("engine - oracle", d))
    print("[stress 1024 NAND, %s] output noise sigma: engine %.5f, oracle %.5f turn (ratio %.4f); "
          "max |noise| engine %.4f, oracle %.4f turn"
          % (form, s_gpu / TURN, s_ref / TURN, s_gpu / s_ref, np.abs(e_gpu).max() / TURN,
             np.abs(e_ref).max() / TURN))
    # 1,024 samples: 2.2 % per sigma; split-FP32 at its fitted split point
    # measured ~4 % above FP64 on 65,536 gates
    assert 0.85 <= s_gpu / s_ref <= 1.2, (s_gpu, s_ref)
    assert abs(d.mean()) <= 5 * d.std() / np.sqrt(len(d))


@pytest.mark.parametrize("form", FORMS)
def test_stress_set_trivial_key_follows_exact_oracle(pkg, oracle, torch_cuda, stress, form):
    """512 NAND gates of the stress set under its trivial key."""
    S = stress
    P = S["P"]
    m = 512
    bk0 = trivial_bootstrapping_key(P, S["lwe"])
    eng = pkg.Engine(pkg.stress_params())
    try:
        eng.upload_bootstrapping_key(bk0, forms=(form,))
        eng.upload_keyswitch_key(S["ks"])
        got = run_gates(torch_cuda, eng, S["gates"][:m], S["ca"][:m], S["cb"][:m], form)
    finally:
        eng.close()
    exact = oracle.boots_gate_exact_batch(P, bk0, S["ks"], S["gates"][:m], S["ca"][:m], S["cb"][:m])
    d = wrap_diff(got, exact)
    print("\n[trivial key, stress 512 NAND, %s] engine - exact: max %d units (2^%.2f), bodies differing %d of %d"
          % (form, np.abs(d).max(), np.log2(np.abs(d).max() + 1), int((d[:, P.n] != 0).sum()), m))
    assert (d[:, :P.n] == 0).all()
    assert np.abs(d).max() <= TRIVIAL_TOL


# ---------------------------------------------------------------------------
# gate outputs against the exact int64 blind rotation (real keys)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("params", ["default", "stress"])
def test_gates_against_exact_int64_bootstrap(pkg, oracle, keys, torch_cuda, stress, params):
    """64 gates per parameter set through the oracle's exact int64 blind
    rotation (no transform at all), the oracle's FFT bootstrap and both
    engine forms.  Reported: each output's phase deviation from the exact
    one.  The engine's deviation must be of the same size as the FFT
    oracle's own (the reference method's), and every bit identical."""
    torch = torch_cuda
    count = 64
    if params == "default":
        P = pyoracle.default_params()
        lwe, ks, bk, bk_fft = keys["lwe"], keys["ks"], keys["bk"], keys["bk_fft"]
        rng = np.random.default_rng(303)
        a = rng.integers(0, 2, count)
        b = rng.integers(0, 2, count)
        gates = np.array(GATE_SET, np.int32)[rng.integers(0, len(GATE_SET), count)]
        oracle.set_seed([303])
        ca = oracle.encrypt_bits(P, a, lwe)
        cb = oracle.encrypt_bits(P, b, lwe)
    else:
        S = stress
        P = S["P"]
        lwe, ks, bk, bk_fft = S["lwe"], S["ks"], S["bk"], S["bk_fft"]
        a, b, gates, ca, cb = S["a"][:count], S["b"][:count], S["gates"][:count], S["ca"][:count], S["cb"][:count]
    truth = gate_truth(gates, a, b)
    exact = oracle.boots_gate_exact_batch(P, bk, ks, gates, ca, cb)
    fft = oracle.boots_gate_batch(P, bk_fft, ks, gates, ca, cb)
    ph_x = oracle.phases(exact, lwe, P.n)
    outs = {"oracle FFT": fft}
    eng = pkg.Engine(pkg.default_params() if params == "default" else pkg.stress_params())
    try:
        eng.upload_bootstrapping_key(bk)
        eng.upload_keyswitch_key(ks)
        for form in FORMS:
            outs["engine " + form] = run_gates(torch, eng, gates, ca, cb, form)
    finally:
        eng.close()
    assert (oracle.decrypt_bits(P, exact, lwe) == truth).all()
    dev_mean = {}
    for name, out in outs.items():
        assert (oracle.decrypt_bits(P, out, lwe) == truth).all(), name
        d = np.abs(wrap_diff(oracle.phases(out, lwe, P.n), ph_x)).astype(np.float64)
        dev_mean[name] = d.mean()
        print("\n[%s set, 64 gates] %s - exact int64: max 2^%.2f mean 2^%.2f turn"
              % (params, name, log2_turn(d.max()), log2_turn(d.mean())), end="")
    print()
    for form in FORMS:
        assert dev_mean["engine " + form] <= 1.6 * dev_mean["oracle FFT"], dev_mean


# ---------------------------------------------------------------------------
# the external-product workload at its full size
# ---------------------------------------------------------------------------
def test_external_products_1024_against_exact(engine, oracle, keys, torch_cuda, P):
    """All 1,024 products of the external-product workload (TRLWE uniform
    int32 from seed 2, TGSW = encryption of X^e with e uniform in [0, 2N)
    from seed 3, built from bootstrapping-key samples of s_i = 1) against
    the exact int64 product, per form: max and rms deviation."""
    torch = torch_cuda
    count = 1024
    rng = np.random.default_rng(2)
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    es = np.random.default_rng(3).integers(0, 2 * P.N, count)
    bkr = keys["bk"].reshape(P.n, P.kpl, 2, P.N)
    base = [bkr[i] for i in np.nonzero(keys["lwe"] == 1)[0][:16]]
    gsw = np.empty((count, P.kpl * 2 * P.N), np.int32)
    for c in range(count):
        g = base[c % len(base)]
        gsw[c] = np.stack([[oracle.mul_by_xai(P.N, int(es[c]), g[p, j]) for j in range(2)]
                           for p in range(P.kpl)]).reshape(-1)
    exact = oracle.extern_mul_exact_batch(P, acc, gsw)
    for form, max_tol, rms_tol in (("fp64", 2, 1.0), ("split_fp32", 2 ** 16, 2 ** 13)):
        nbytes = engine.tgsw_fft_bytes(form)
        d_gsw = torch.zeros(count * nbytes, dtype=torch.uint8, device="cuda")
        engine.tgsw_to_fft(dev(torch, gsw), d_gsw, count, form, stream=cur(torch))
        d_acc = dev(torch, acc)
        engine.tGswFFTExternMulToTLwe(d_acc, d_gsw, count, form, stream=cur(torch))
        torch.cuda.synchronize()
        engine.synchronize()
        d = wrap_diff(d_acc.cpu().numpy(), exact).astype(np.float64)
        rms = float(np.sqrt((d ** 2).mean()))
        print("\n[external products 1024, %s] vs exact int64: max %d units (2^%.2f turn), rms %.3f units "
              "(2^%.2f turn), words exact %.4f" % (form, np.abs(d).max(), log2_turn(np.abs(d).max()), rms,
                                                  log2_turn(rms), float((d == 0).mean())))
        assert np.abs(d).max() <= max_tol
        assert rms <= rms_tol


# ---------------------------------------------------------------------------
# the paths either side of the gate bootstrap at size: bootsMUX and the
# programmable bootstrap, default set, both forms
# ---------------------------------------------------------------------------
def noise_stats_check(tag, form, d, e_gpu, e_ref, sigma_tol):
    """Print and check the engine-vs-oracle phase statistics of one workload:
    the same noise sigma within sampling error, no bias, no heavier tail."""
    s_gpu, s_ref, s_d = e_gpu.std(), e_ref.std(), d.std()
    print("\n[%s, %s] " % (tag, form) + describe("engine - oracle", d))
    print("[%s, %s] output noise sigma: engine 2^%.3f, oracle 2^%.3f turn (ratio %.4f); max |noise| engine "
          "2^%.2f, oracle 2^%.2f" % (tag, form, log2_turn(s_gpu), log2_turn(s_ref), s_gpu / s_ref,
                                     log2_turn(np.abs(e_gpu).max()), log2_turn(np.abs(e_ref).max())))
    assert 1 - sigma_tol <= s_gpu / s_ref <= 1 + sigma_tol, (s_gpu, s_ref)
    assert abs(d.mean()) <= 5 * s_d / np.sqrt(len(d))
    assert s_d <= (1 + sigma_tol) * np.hypot(s_gpu, s_ref)
    assert np.abs(e_gpu).max() <= 1.25 * max(np.abs(e_ref).max(), 6 * s_ref)
    assert np.abs(d).max() < 2 ** 28


@pytest.fixture(scope="module")
def mux_set(oracle, keys, P):
    """1,024 bootsMUX (2,048 bootstraps) on random select/input bits, and the
    oracle's on every host thread."""
    rng = np.random.default_rng(41)
    count = 1024
    bits = rng.integers(0, 2, (3, count))
    oracle.set_seed([41])
    enc = [oracle.encrypt_bits(P, bits[i], keys["lwe"]) for i in range(3)]
    ref = oracle.boots_mux_batch(P, keys["bk_fft"], keys["ks"], enc[0], enc[1], enc[2])
    return {"enc": enc, "ref": ref, "truth": np.where(bits[0] == 1, bits[1], bits[2])}


@pytest.mark.parametrize("form", FORMS)
def test_mux_1024_against_oracle(engine, oracle, keys, torch_cuda, P, mux_set, form):
    """All 1,024 MUX outputs decrypt like the oracle's and the truth, with the
    oracle's output-noise distribution (sigma within 12 %: 1,024 samples)."""
    torch = torch_cuda
    count = len(mux_set["truth"])
    e = mux_set["enc"]
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    engine.bootsMUX(d_out, dev(torch, e[0]), dev(torch, e[1]), dev(torch, e[2]), count, form, stream=cur(torch))
    torch.cuda.synchronize()
    engine.synchronize()
    got = d_out.cpu().numpy()
    bits = oracle.decrypt_bits(P, got, keys["lwe"])
    ref_bits = oracle.decrypt_bits(P, mux_set["ref"], keys["lwe"])
    assert (ref_bits == mux_set["truth"]).all()
    assert (bits == mux_set["truth"]).all(), int((bits != mux_set["truth"]).sum())
    ph = oracle.phases(got, keys["lwe"], P.n)
    ph_ref = oracle.phases(mux_set["ref"], keys["lwe"], P.n)
    noise_stats_check("bootsMUX 1024", form, wrap_diff(ph, ph_ref).astype(np.float64), output_noise(ph, bits),
                      output_noise(ph_ref, ref_bits), 0.12)


LUT_P = 8  # messages of the lookup-table workload (padded: phase m / 16)


def lut_decode(phases, p):
    """Padded message of Torus32 phases: round(phase * 2p) mod 2p."""
    ph = np.asarray(phases, np.int64) & 0xFFFFFFFF
    return ((ph * 2 * p + (1 << 31)) >> 32) % (2 * p)


@pytest.fixture(scope="module")
def lut_set(pkg, oracle, keys, P):
    """1,024 programmable bootstraps of random messages m < 8 through the
    table f(m) = 5m + 3 mod 8, and the oracle's on every host thread."""
    rng = np.random.default_rng(43)
    count = 1024
    m = rng.integers(0, LUT_P, count)
    f = (5 * np.arange(LUT_P) + 3) % LUT_P
    table = np.array([pkg.mod_switch_to_torus32(int(v), 2 * LUT_P) for v in f], np.int32)
    tv = oracle.test_vector(P.N, table)
    pkg.set_seed([43])
    x = pkg.encrypt_phases(P, [pkg.mod_switch_to_torus32(int(v), 2 * LUT_P) for v in m], keys["lwe"])
    ref = oracle.bootstrap_tv_batch(P, keys["bk_fft"], keys["ks"], tv, x)
    ideal = np.array([pkg.mod_switch_to_torus32(int(v), 2 * LUT_P) for v in f[m]], np.int64)
    return {"x": x, "tv": tv, "ref": ref, "want": f[m], "ideal": ideal}


@pytest.mark.parametrize("form", FORMS)
def test_lookup_table_1024_against_oracle(engine, oracle, keys, torch_cuda, P, lut_set, form):
    """All 1,024 programmable bootstraps decode to the table's value, like the
    oracle's, with the oracle's output-noise distribution."""
    torch = torch_cuda
    count = len(lut_set["want"])
    d_x = dev(torch, lut_set["x"])
    d_out = torch.zeros_like(d_x)
    engine.bootstrap_tv(d_out, d_x, dev(torch, lut_set["tv"]), count, form, stream=cur(torch))
    torch.cuda.synchronize()
    engine.synchronize()
    got = d_out.cpu().numpy()
    ph = oracle.phases(got, keys["lwe"], P.n)
    ph_ref = oracle.phases(lut_set["ref"], keys["lwe"], P.n)
    assert (lut_decode(ph_ref, LUT_P) == lut_set["want"]).all()
    assert (lut_decode(ph, LUT_P) == lut_set["want"]).all()
    e_gpu = wrap_diff(ph, lut_set["ideal"]).astype(np.float64)
    e_ref = wrap_diff(ph_ref, lut_set["ideal"]).astype(np.float64)
    noise_stats_check("lookup table 1024", form, wrap_diff(ph, ph_ref).astype(np.float64), e_gpu, e_ref, 0.12)
