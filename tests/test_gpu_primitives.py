"""GPU parity of the building blocks, through the C ABI, against the oracle.

Bit-exact: X^a - 1 rotation, sample extraction, key switching (integer work).
Tolerances (Torus32 units, 2^32 = one turn):
  * Lagrange processor, FP64: relative 1e-9 against the oracle's 2N-point
    transform; Lagrange -> torus within 1 unit (truncating conversion);
  * external product against the exact int64 negacyclic product:
    FP64 form |err| <= 2 units; split-FP32 form |err| <= 2^16 units
    (measured rms ~2^11 for the default set, split point s = 24).
"""
import numpy as np
import pytest

from helpers import wrap_diff

pytestmark = pytest.mark.gpu

EP_TOL = {"fp64": 2, "split_fp32": 2 ** 16}


def dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def sync(torch):
    torch.cuda.synchronize()


def cur(torch):
    return torch.cuda.current_stream().cuda_stream


def test_lagrange_processor(engine, oracle, torch_cuda, P):
    torch = torch_cuda
    rng = np.random.default_rng(31)
    count = 9
    ints = rng.integers(-64, 64, (count, P.N)).astype(np.int32)
    tors = rng.integers(-2 ** 31, 2 ** 31, (count, P.N)).astype(np.int32)
    d_out = torch.zeros((count, P.N), dtype=torch.float64, device="cuda")
    engine.IntPolynomial_ifft(dev(torch, ints), d_out, count, stream=cur(torch))
    sync(torch)
    got = host(d_out)
    for c in range(count):
        want = oracle.int_poly_ifft(P.N, ints[c])
        g = got[c, 0::2] + 1j * got[c, 1::2]
        assert np.abs(g - want).max() <= 1e-9 * np.abs(want).max()
    engine.TorusPolynomial_ifft(dev(torch, tors), d_out, count, stream=cur(torch))
    sync(torch)
    lag = host(d_out)
    for c in range(count):
        want = oracle.torus_poly_ifft(P.N, tors[c])
        g = lag[c, 0::2] + 1j * lag[c, 1::2]
        assert np.abs(g - want).max() <= 1e-9 * np.abs(want).max()
    # back to the torus: the round trip reproduces the polynomial up to the
    # truncating conversion
    d_back = torch.zeros((count, P.N), dtype=torch.int32, device="cuda")
    engine.TorusPolynomial_fft(d_out, d_back, count, stream=cur(torch))
    sync(torch)
    back = host(d_back)
    assert np.abs(wrap_diff(back, tors)).max() <= 1
    for c in range(2):
        want = oracle.torus_poly_fft(P.N, lag[c, 0::2] + 1j * lag[c, 1::2])
        assert np.abs(wrap_diff(back[c], want)).max() <= 1
    # pointwise multiply-accumulate
    a = rng.standard_normal((count, P.N))
    b = rng.standard_normal((count, P.N))
    acc = rng.standard_normal((count, P.N))
    d_acc = dev(torch, acc)
    engine.LagrangeHalfCPolynomialAddMul(d_acc, dev(torch, a), dev(torch, b), count, stream=cur(torch))
    sync(torch)
    ca = a[:, 0::2] + 1j * a[:, 1::2]
    cb = b[:, 0::2] + 1j * b[:, 1::2]
    want = acc[:, 0::2] + 1j * acc[:, 1::2] + ca * cb
    g = host(d_acc)
    assert np.allclose(g[:, 0::2] + 1j * g[:, 1::2], want, rtol=1e-12, atol=1e-12)


def test_lagrange_matches_reference_convention(engine, torch_cuda, P):
    """Values are P(w^(2m+1)), w = e^{i pi/N} (tGswFFTExternMulToTLwe.cpp:97-130)."""
    torch = torch_cuda
    rng = np.random.default_rng(32)
    c = rng.integers(-64, 64, P.N).astype(np.int32)
    d_out = torch.zeros((1, P.N), dtype=torch.float64, device="cuda")
    engine.IntPolynomial_ifft(dev(torch, c[None]), d_out, 1, stream=cur(torch))
    sync(torch)
    got = host(d_out)[0]
    w = np.exp(1j * np.pi * (2 * np.arange(P.N // 2) + 1) / P.N)
    want = np.array([np.polyval(c[::-1].astype(np.float64), wi) for wi in w])
    assert np.abs(got[0::2] + 1j * got[1::2] - want).max() < 1e-7 * np.abs(want).max()


@pytest.mark.parametrize("a_vals", [[0, 1, 5, 1023, 1024, 1027, 2047]])
def test_mul_by_xai_minus_one_bit_exact(engine, oracle, torch_cuda, P, a_vals):
    torch = torch_cuda
    rng = np.random.default_rng(33)
    count = len(a_vals)
    x = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    d_out = torch.zeros_like(dev(torch, x))
    engine.tLweMulByXaiMinusOne(d_out, dev(torch, np.array(a_vals, np.int32)), dev(torch, x), count,
                                stream=cur(torch))
    sync(torch)
    got = host(d_out)
    for c, a in enumerate(a_vals):
        for j in range(2):
            want = oracle.mul_by_xai_minus_one(P.N, a, x[c, j * P.N:(j + 1) * P.N])
            assert (got[c, j * P.N:(j + 1) * P.N] == want).all()


def test_extract_bit_exact(engine, oracle, torch_cuda, P):
    torch = torch_cuda
    rng = np.random.default_rng(34)
    count = 5
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    d_out = torch.zeros((count, P.N + 1), dtype=torch.int32, device="cuda")
    engine.tLweExtractLweSample(d_out, dev(torch, acc), count, stream=cur(torch))
    sync(torch)
    got = host(d_out)
    for c in range(count):
        assert (got[c] == oracle.extract(P, acc[c])).all()


@pytest.mark.parametrize("count", [1, 7, 8, 9, 33, 37, 1217, 5000])
def test_keyswitch_bit_exact(engine, oracle, keys, torch_cuda, P, count):
    """The key switch (shared-memory ring kernel) against the oracle: batch
    sizes below one CTA, uneven sub-groups (1217 = 152 CTAs of 8-9), and more
    than 32 per SM (5000: 157 CTAs of 32, a second wave); for the large
    batches every 97th ciphertext plus the first and last are checked."""
    torch = torch_cuda
    rng = np.random.default_rng(35 + count)
    u = rng.integers(-2 ** 31, 2 ** 31, (count, P.N + 1)).astype(np.int32)
    d_out = torch.zeros((count, P.n + 1), dtype=torch.int32, device="cuda")
    engine.lweKeySwitch(d_out, dev(torch, u), count, stream=cur(torch))
    sync(torch)
    engine.synchronize()
    got = host(d_out)
    check = range(count) if count <= 64 else sorted(set(range(0, count, 97)) | {count - 1, 31, 32})
    for c in check:
        assert (got[c] == oracle.keyswitch(P, keys["ks"], u[c])).all()


def _tgsw_monomials(oracle, P, es, tlwe_key, seed):
    """TGSW encryptions of X^e (encrypt 1, rotate every row by X^e)."""
    oracle.set_seed([seed])
    out = []
    for e in es:
        g = oracle.tgsw_encrypt_int(P, 1, P.tlwe_alpha, tlwe_key).reshape(P.kpl, P.k + 1, P.N)
        g = np.stack([[oracle.mul_by_xai(P.N, int(e), g[p, j]) for j in range(P.k + 1)]
                      for p in range(P.kpl)])
        out.append(g.reshape(-1))
    return np.stack(out)


@pytest.mark.parametrize("form", ["fp64", "split_fp32"])
def test_external_product_vs_exact(engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    rng = np.random.default_rng(40)
    count = 12
    es = rng.integers(0, 2 * P.N, count)
    gsw = _tgsw_monomials(oracle, P, es, keys["tlwe"], 41)
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    nbytes = engine.tgsw_fft_bytes(form)
    d_gsw = torch.zeros(count * nbytes, dtype=torch.uint8, device="cuda")
    engine.tgsw_to_fft(dev(torch, gsw), d_gsw, count, form, stream=cur(torch))
    d_acc = dev(torch, acc)
    engine.tGswFFTExternMulToTLwe(d_acc, d_gsw, count, form, per_item=True, stream=cur(torch))
    sync(torch)
    got = host(d_acc)
    for c in range(count):
        exact = oracle.extern_mul_exact(P, acc[c], gsw[c])
        err = np.abs(wrap_diff(got[c], exact)).max()
        assert err <= EP_TOL[form], (form, c, err)
    # one TGSW shared by all items
    d_acc = dev(torch, acc)
    engine.tGswFFTExternMulToTLwe(d_acc, d_gsw, count, form, per_item=False, stream=cur(torch))
    sync(torch)
    got = host(d_acc)
    for c in (0, count - 1):
        exact = oracle.extern_mul_exact(P, acc[c], gsw[0])
        assert np.abs(wrap_diff(got[c], exact)).max() <= EP_TOL[form]


@pytest.mark.parametrize("form", ["fp64", "split_fp32"])
def test_mux_rotate_vs_exact(engine, oracle, keys, torch_cuda, P, form):
    torch = torch_cuda
    rng = np.random.default_rng(42)
    count = 6
    bits = rng.integers(0, 2, count)
    oracle.set_seed([43])
    gsw = np.stack([oracle.tgsw_encrypt_int(P, int(b), P.tlwe_alpha, keys["tlwe"]) for b in bits])
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    barai = np.array([0, 1, 513, 1024, 1500, 2047], np.int32)
    nbytes = engine.tgsw_fft_bytes(form)
    d_gsw = torch.zeros(count * nbytes, dtype=torch.uint8, device="cuda")
    engine.tgsw_to_fft(dev(torch, gsw), d_gsw, count, form, stream=cur(torch))
    d_res = torch.zeros((count, 2 * P.N), dtype=torch.int32, device="cuda")
    engine.tfhe_MuxRotate_FFT(d_res, dev(torch, acc), d_gsw, dev(torch, barai), count, form,
                              stream=cur(torch))
    sync(torch)
    got = host(d_res)
    for c in range(count):
        if barai[c] == 0:
            assert (got[c] == acc[c]).all()
            continue
        rot = np.concatenate([oracle.mul_by_xai_minus_one(P.N, int(barai[c]), acc[c, j * P.N:(j + 1) * P.N])
                              for j in range(2)])
        want = oracle.extern_mul_exact(P, rot, gsw[c]).astype(np.int64) + acc[c]
        assert np.abs(wrap_diff(got[c], want)).max() <= EP_TOL[form]


def test_external_product_exactness_statistics(engine, oracle, keys, torch_cuda, P):
    """Deviation of each form from the exact int64 product (reported in the
    test log): FP64 within a unit or two, split-FP32 near 2^-21 of a turn."""
    torch = torch_cuda
    rng = np.random.default_rng(44)
    count = 16
    gsw = _tgsw_monomials(oracle, P, rng.integers(0, 2 * P.N, count), keys["tlwe"], 45)
    acc = rng.integers(-2 ** 31, 2 ** 31, (count, 2 * P.N)).astype(np.int32)
    exact = np.stack([oracle.extern_mul_exact(P, acc[c], gsw[c]) for c in range(count)])
    for form, rms_bound in (("fp64", 1.0), ("split_fp32", 2 ** 13)):
        nbytes = engine.tgsw_fft_bytes(form)
        d_gsw = torch.zeros(count * nbytes, dtype=torch.uint8, device="cuda")
        engine.tgsw_to_fft(dev(torch, gsw), d_gsw, count, form, stream=cur(torch))
        d_acc = dev(torch, acc)
        engine.tGswFFTExternMulToTLwe(d_acc, d_gsw, count, form, stream=cur(torch))
        sync(torch)
        d = wrap_diff(host(d_acc), exact).astype(np.float64)
        rms = float(np.sqrt((d ** 2).mean()))
        print("external product %s vs exact: max %d rms %.2f units (2^%.1f turn)"
              % (form, np.abs(d).max(), rms, np.log2(max(rms, 1e-9)) - 32))
        assert rms <= rms_bound


def test_bootstrapping_key_import_reference_format(pkg, keys, oracle, torch_cuda, P):
    """A key uploaded in the reference's transform format (TGswSampleFFT
    layout) is recovered exactly: gates give bit-identical ciphertexts to the
    time-domain upload."""
    torch = torch_cuda
    e1 = pkg.Engine(pkg.default_params())
    e2 = pkg.Engine(pkg.default_params())
    try:
        e1.upload_bootstrapping_key(keys["bk"])
        e2.upload_bootstrapping_key_fft(keys["bk_fft"])
        for e in (e1, e2):
            e.upload_keyswitch_key(keys["ks"])
        rng = np.random.default_rng(46)
        oracle.set_seed([47])
        ca = oracle.encrypt_bits(P, rng.integers(0, 2, 4), keys["lwe"])
        cb = oracle.encrypt_bits(P, rng.integers(0, 2, 4), keys["lwe"])
        for form in ("fp64", "split_fp32"):
            outs = []
            for e in (e1, e2):
                d_out = torch.zeros((4, P.n + 1), dtype=torch.int32, device="cuda")
                e.bootsGate("NAND", d_out, dev(torch, ca), dev(torch, cb), 4, form, stream=cur(torch))
                sync(torch)
                outs.append(host(d_out))
            assert (outs[0] == outs[1]).all()
    finally:
        e1.close()
        e2.close()
