"""The upstream TFHE API over the engine (include/tfhe/tfhe.h, tfhe_io.h):
C programs written against <tfhe/tfhe.h> compile with `-I include`, link
with libtfhe_gb300.so and run.

CPU: tests/compat/roundtrip.c's client step (keygen, encryption, file
export) reproduces the engine's and the oracle's keys and ciphertexts; the
reference's own test bench (test_bench/client/alice.c, client/verify.c,
server/cloud.c) compiles unchanged against these headers, alice and verify
run, and with the oracle standing in for the cloud (16 OR gates) verify
prints 499 | 388 = 503 -- the test bench's known answer.
GPU: the whole round trip of roundtrip.c (client, cloud on the GPU through
every gate function, verifier) decrypts every result to its plaintext.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from oracle import pyoracle
from oracle.ref_pin import build_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def _build(pkg, src, out):
    libdir = os.path.dirname(pkg.LIB_PATH)
    cmd = [_cc(), "-O1", "-std=gnu11", "-Wall", "-I", os.path.join(ROOT, "include"), src, "-o", out,
           "-L", libdir, "-ltfhe_gb300", "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run(args, cwd=None, timeout=600):
    r = subprocess.run(args, capture_output=True, text=True, cwd=cwd, timeout=timeout)
    return r.returncode, r.stdout + r.stderr


def test_roundtrip_client_step_cpu(pkg, oracle, tmp_path):
    exe = _build(pkg, os.path.join(HERE, "compat", "roundtrip.c"), str(tmp_path / "roundtrip"))
    rc, log = _run([exe, str(tmp_path), "client", "499", "388"])
    assert rc == 0, log
    kinds = [k for k, _ in pkg.keyfile_records(str(tmp_path / "secret.key"))]
    assert kinds == [pkg.KEYFILE_SECRET_KEY]
    assert [k for k, _ in pkg.keyfile_records(str(tmp_path / "cloud.key"))] == [pkg.KEYFILE_CLOUD_KEY]
    P, lwe, tlwe, bk, ks = pkg.load_secret_key(str(tmp_path / "secret.key"))
    # the keys are new_random_gate_bootstrapping_secret_keyset after seeding {27, 18, 28}
    want = oracle.gate_keyset(pyoracle.default_params(), [27, 18, 28])
    for got, w in zip((lwe, tlwe, ks, bk), want):
        assert (got == w).all()
    P2, bk2, ks2 = pkg.load_cloud_key(str(tmp_path / "cloud.key"))
    assert (bk2 == bk).all() and (ks2 == ks).all() and P2.n == P.n
    ct = pkg.load_ciphertexts(str(tmp_path / "cloud.data"))
    assert ct.shape == (32, P.n + 1)
    bits = pkg.decrypt_bits(P, ct, lwe)
    assert [int(b) for b in bits] == [(499 >> i) & 1 for i in range(16)] + [(388 >> i) & 1 for i in range(16)]


@pytest.mark.skipif(not os.path.isdir(os.path.join(build_ref.REF, "test_bench")),
                    reason="reference sources not present")
def test_reference_test_bench_against_compat_headers(pkg, oracle, tmp_path):
    """alice.c, cloud.c, verify.c of the reference, unmodified, built against
    include/tfhe; alice and verify run (no GPU needed); the oracle computes the
    cloud's 16 OR gates from alice's files."""
    tb = os.path.join(build_ref.REF, "test_bench")
    exes = {}
    for name, rel in (("alice", "client/alice.c"), ("verify", "client/verify.c"), ("cloud", "server/cloud.c")):
        exes[name] = _build(pkg, os.path.join(tb, rel), str(tmp_path / name))
    work = tmp_path / "run"
    (work / "keys").mkdir(parents=True)
    (work / "data").mkdir()
    rc, log = _run([exes["alice"]], cwd=str(work))
    assert rc == 0, log
    P, lwe, tlwe, bk, ks = pkg.load_secret_key(str(work / "keys" / "secret.key"))
    OP = pyoracle.default_params()
    want = oracle.gate_keyset(OP, [314, 1592, 657])  # alice.c:15-16
    for got, w in zip((lwe, tlwe, ks, bk), want):
        assert (got == w).all()
    ct = pkg.load_ciphertexts(str(work / "data" / "cloud.data"))
    assert [int(b) for b in pkg.decrypt_bits(P, ct, lwe)] == \
        [(499 >> i) & 1 for i in range(16)] + [(388 >> i) & 1 for i in range(16)]
    # the cloud step (cloud.c:58-62: bootsOR bit by bit) on the oracle
    _, cbk, cks = pkg.load_cloud_key(str(work / "keys" / "cloud.key"))
    out = oracle.boots_gate_batch(OP, oracle.bk_to_fft(OP, cbk), cks, np.full(16, pyoracle.GATES["OR"]),
                                  ct[:16], ct[16:])
    answer = work / "data" / "answer.data"
    for i in range(16):
        pkg.save_ciphertexts(str(answer), P, out[i:i + 1], append=i > 0)
    rc, log = _run([exes["verify"]], cwd=str(work))
    assert rc == 0, log
    m = re.search(r"And the result is: (-?\d+) vs (\d+)", log)
    assert m and int(m.group(1)) == int(m.group(2)) == (499 | 388), log


@pytest.mark.gpu
@pytest.mark.skipif(not os.path.isdir(os.path.join(build_ref.REF, "test_bench")),
                    reason="reference test bench not present (TFHE_REFERENCE_DIR)")
def test_reference_cloud_runs_its_gates_on_gpu(pkg, tmp_path):
    """The reference's own test bench end to end with the cloud on the GPU:
    alice.c, cloud.c and verify.c, unmodified, built against include/tfhe
    and linked with this library.  alice writes the keys and the two
    encrypted 16-bit numbers; cloud (cloud.c:39-74) reads them and runs its
    16 bootsOR calls (cloud.c:58-62) -- each one a gate bootstrap on the GPU,
    shown by the library's per-call trace -- and writes answer.data; verify
    decrypts it and prints 499 | 388 = 503."""
    tb = os.path.join(build_ref.REF, "test_bench")
    exes = {}
    for name, rel in (("alice", "client/alice.c"), ("verify", "client/verify.c"), ("cloud", "server/cloud.c")):
        exes[name] = _build(pkg, os.path.join(tb, rel), str(tmp_path / name))
    work = tmp_path / "run"
    (work / "keys").mkdir(parents=True)
    (work / "data").mkdir()
    rc, log_a = _run([exes["alice"]], cwd=str(work))
    assert rc == 0, log_a
    env = dict(os.environ, TFHE_GB300_TRACE="1")
    r = subprocess.run([exes["cloud"]], capture_output=True, text=True, cwd=str(work), timeout=600, env=env)
    log_c = r.stdout + r.stderr
    assert r.returncode == 0, log_c
    trace = [ln for ln in log_c.splitlines() if ln.startswith("tfhe_gb300 trace: bootsOR: 1 sample(s) on GPU 0")]
    assert len(trace) == 16, log_c
    rc, log_v = _run([exes["verify"]], cwd=str(work))
    assert rc == 0, log_v
    print("\n---- alice ----\n" + log_a + "\n---- cloud (TFHE_GB300_TRACE=1) ----\n" + log_c +
          "\n---- verify ----\n" + log_v)
    m = re.search(r"And the result is: (-?\d+) vs (\d+)", log_v)
    assert m and int(m.group(1)) == int(m.group(2)) == (499 | 388), log_v


@pytest.mark.gpu
def test_roundtrip_on_gpu(pkg, tmp_path):
    exe = _build(pkg, os.path.join(HERE, "compat", "roundtrip.c"), str(tmp_path / "roundtrip"))
    for x, y in ((499, 388), (65535, 1), (12345, 54321)):
        d = tmp_path / ("r%d_%d" % (x, y))
        d.mkdir()
        rc, log = _run([exe, str(d), "all", str(x), str(y)])
        assert rc == 0, log
        assert "WRONG" not in log and log.count("result") == 18, log
