"""Host-side binding of the GB300 TFHE engine (ctypes over include/tfhe_gpu.h).

This mirrors the reference's operator interface for the bootstrapping path
(kernel/src/include/fpga_constants.h:57-69, the upstream gate calls of
test_bench/server/cloud.c:10-35): one method per C entry point, same names,
device-batch forms over device buffers (any object with a data_ptr(), e.g.
torch tensors, or raw integer addresses) and host-buffer forms over numpy
arrays.  Errors raise TfheError carrying the status and the context's
last_error; there is no CPU fallback -- if the shared library is missing the
import fails loudly.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtfhe_gb300.so")

I32P = ctypes.POINTER(ctypes.c_int32)
U32P = ctypes.POINTER(ctypes.c_uint32)
F64P = ctypes.POINTER(ctypes.c_double)
VP = ctypes.c_void_p

FP64 = 0
SPLIT_FP32 = 1
FORMS = {"fp64": FP64, "split_fp32": SPLIT_FP32}

GATES = {"NAND": 0, "AND": 1, "OR": 2, "XOR": 3, "XNOR": 4, "NOR": 5,
         "ANDNY": 6, "ANDYN": 7, "ORNY": 8, "ORYN": 9}

STATUS = {0: "ok", 1: "bad parameter", 2: "out of memory", 3: "timeout",
          4: "device error", 5: "key not uploaded"}


class TfheError(RuntimeError):
    def __init__(self, status, detail):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "?"), status, detail))
        self.status = status


class Params(ctypes.Structure):
    """tfhe_params (include/tfhe_gpu.h)."""
    _fields_ = [("n", ctypes.c_int32), ("N", ctypes.c_int32), ("k", ctypes.c_int32),
                ("l", ctypes.c_int32), ("Bgbit", ctypes.c_int32), ("ks_t", ctypes.c_int32),
                ("ks_basebit", ctypes.c_int32), ("split_bits", ctypes.c_int32),
                ("lwe_alpha", ctypes.c_double), ("tlwe_alpha", ctypes.c_double)]

    @property
    def kpl(self):
        return (self.k + 1) * self.l

    def tgsw_words(self):
        return self.kpl * (self.k + 1) * self.N

    def ks_words(self):
        return self.k * self.N * self.ks_t * (1 << self.ks_basebit) * (self.n + 1)


def measure_fp32_peak(device=0, iters=65536):
    """Measured FP32 FMA-pipe peak of the device: (TFLOP/s, probe ms)."""
    tf, ms = ctypes.c_double(), ctypes.c_double()
    st = lib().tfhe_gpu_measure_fp32_peak(int(device), int(iters), ctypes.byref(tf), ctypes.byref(ms))
    if st:
        raise TfheError(st, "measure_fp32_peak")
    return tf.value, ms.value


def measure_fp64_peak(device=0, iters=2048):
    """Measured FP64 FMA-pipe peak of the device: (TFLOP/s, probe ms)."""
    tf, ms = ctypes.c_double(), ctypes.c_double()
    st = lib().tfhe_gpu_measure_fp64_peak(int(device), int(iters), ctypes.byref(tf), ctypes.byref(ms))
    if st:
        raise TfheError(st, "measure_fp64_peak")
    return tf.value, ms.value


def default_params():
    """The reference's default gate set (constants.h:26-40)."""
    return Params(n=630, N=1024, k=1, l=3, Bgbit=7, ks_t=8, ks_basebit=2, split_bits=0,
                  lwe_alpha=2.0 ** -15, tlwe_alpha=2.0 ** -25)


def stress_params():
    """Alternative set: n=500, l=2, Bgbit=10, LWE 2^-15, TRLWE 2^-24."""
    return Params(n=500, N=1024, k=1, l=2, Bgbit=10, ks_t=8, ks_basebit=2, split_bits=0,
                  lwe_alpha=2.0 ** -15, tlwe_alpha=2.0 ** -24)


# Every symbol of include/tfhe_gpu.h with its ctypes signature.
SIGNATURES = {
    "tfhe_gpu_default_params": (None, [ctypes.c_void_p]),
    "tfhe_gpu_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(VP)]),
    "tfhe_gpu_destroy": (None, [VP]),
    "tfhe_gpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "tfhe_gpu_last_error": (ctypes.c_char_p, [VP]),
    "tfhe_gpu_get_params": (ctypes.c_int, [VP, ctypes.c_void_p]),
    "tfhe_gpu_stream": (VP, [VP]),
    "tfhe_gpu_synchronize": (ctypes.c_int, [VP]),
    "tfhe_gpu_tgsw_fft_bytes": (ctypes.c_size_t, [VP, ctypes.c_int]),
    "tfhe_gpu_device_bytes": (ctypes.c_size_t, [VP]),
    "tfhe_gpu_set_groups_per_cta": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int32]),
    "tfhe_gpu_get_groups_per_cta": (ctypes.c_int32, [VP, ctypes.c_int]),
    "tfhe_gpu_upload_bootstrapping_key": (ctypes.c_int, [VP, I32P, ctypes.c_uint32]),
    "tfhe_gpu_upload_bootstrapping_key_fft": (ctypes.c_int, [VP, F64P, ctypes.c_uint32]),
    "tfhe_gpu_upload_keyswitch_key": (ctypes.c_int, [VP, I32P]),
    "tfhe_gpu_tgsw_to_fft": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, ctypes.c_int, VP]),
    "tfhe_gpu_IntPolynomial_ifft": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_TorusPolynomial_ifft": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_TorusPolynomial_fft": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_LagrangeHalfCPolynomialAddMul": (ctypes.c_int, [VP, VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_tLweMulByXaiMinusOne": (ctypes.c_int, [VP, VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_tGswFFTExternMulToTLwe": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, ctypes.c_int32,
                                                       ctypes.c_int, VP]),
    "tfhe_gpu_tfhe_MuxRotate_FFT": (ctypes.c_int, [VP, VP, VP, VP, ctypes.c_int32, VP,
                                                   ctypes.c_int32, ctypes.c_int, VP]),
    "tfhe_gpu_tfhe_blindRotate_FFT": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, ctypes.c_int, VP]),
    "tfhe_gpu_tLweExtractLweSample": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_lweKeySwitch": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, VP]),
    "tfhe_gpu_tfhe_bootstrap_woKS_FFT": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, ctypes.c_int32,
                                                        ctypes.c_int, VP]),
    "tfhe_gpu_tfhe_bootstrap_FFT": (ctypes.c_int, [VP, VP, VP, ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.c_int, VP]),
    "tfhe_gpu_bootsGate": (ctypes.c_int, [VP, ctypes.c_int32, VP, VP, VP, ctypes.c_int32,
                                          ctypes.c_int, VP]),
    "tfhe_gpu_bootsGates": (ctypes.c_int, [VP, VP, VP, VP, VP, ctypes.c_int32, ctypes.c_int, VP]),
    "tfhe_gpu_bootsMUX": (ctypes.c_int, [VP, VP, VP, VP, VP, ctypes.c_int32, ctypes.c_int, VP]),
    "tfhe_gpu_bootsGates_host": (ctypes.c_int, [VP, I32P, ctypes.c_int32, I32P, I32P, I32P,
                                                ctypes.c_int32, ctypes.c_int]),
    "tfhe_gpu_bootsGates_host_split": (ctypes.c_int, [ctypes.POINTER(VP), ctypes.c_int32, I32P, ctypes.c_int32,
                                                      I32P, I32P, I32P, ctypes.c_int32, ctypes.c_int]),
    "tfhe_gpu_bootsGates_noalloc": (ctypes.c_int, [VP, VP, VP, VP, VP, ctypes.c_int32, ctypes.c_int,
                                                   VP]),
    "tfhe_gpu_server_create": (ctypes.c_int, [VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int,
                                               ctypes.POINTER(VP)]),
    "tfhe_gpu_server_destroy": (None, [VP]),
    "tfhe_gpu_server_last_error": (ctypes.c_char_p, [VP]),
    "tfhe_gpu_server_submit": (ctypes.c_int, [VP, I32P, ctypes.c_int32, ctypes.c_int32, I32P, I32P,
                                               ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]),
    "tfhe_gpu_server_step": (ctypes.c_int, [VP, I32P]),
    "tfhe_gpu_server_poll": (ctypes.c_int, [VP, ctypes.c_int64, I32P, I32P,
                                             ctypes.POINTER(ctypes.c_double)]),
    "tfhe_gpu_server_stats": (ctypes.c_int, [VP, F64P, F64P, F64P, ctypes.POINTER(ctypes.c_int64)]),
    "tfhe_gpu_upload_cloud_key": (ctypes.c_int, [VP, I32P, I32P, ctypes.c_uint32]),
    "tfhe_gpu_bootsMUX_host": (ctypes.c_int, [VP, I32P, I32P, I32P, I32P, ctypes.c_int32, ctypes.c_int]),
    "tfhe_gpu_upload_cloud_key_file": (ctypes.c_int, [VP, ctypes.c_char_p, ctypes.c_uint32]),
    "tfhe_keyfile_bk_words": (ctypes.c_int64, [ctypes.c_void_p]),
    "tfhe_keyfile_ks_words": (ctypes.c_int64, [ctypes.c_void_p]),
    "tfhe_keyfile_peek": (ctypes.c_int, [VP, I32P, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "tfhe_keyfile_write_params": (ctypes.c_int, [VP, ctypes.c_void_p]),
    "tfhe_keyfile_write_cloud_key": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, I32P]),
    "tfhe_keyfile_write_secret_key": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, I32P, I32P, I32P]),
    "tfhe_keyfile_write_ciphertexts": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, F64P, ctypes.c_int64]),
    "tfhe_keyfile_read_params": (ctypes.c_int, [VP, ctypes.c_void_p]),
    "tfhe_keyfile_read_cloud_key": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, I32P]),
    "tfhe_keyfile_read_secret_key": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, I32P, I32P, I32P]),
    "tfhe_keyfile_read_ciphertexts": (ctypes.c_int, [VP, ctypes.c_void_p, I32P, F64P,
                                                     ctypes.POINTER(ctypes.c_int64)]),
    "tfhe_keyfile_save_cloud_key": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, I32P, I32P]),
    "tfhe_keyfile_load_cloud_key": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, I32P, I32P]),
    "tfhe_gpu_graph_gates_create": (ctypes.c_int, [VP, VP, ctypes.c_int32, VP, VP, VP, ctypes.c_int32,
                                                   ctypes.c_int, ctypes.POINTER(VP)]),
    "tfhe_gpu_graph_launch": (ctypes.c_int, [VP, VP]),
    "tfhe_gpu_graph_kernel_count": (ctypes.c_int32, [VP]),
    "tfhe_gpu_graph_destroy": (None, [VP]),
    "tfhe_gpu_autotune": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int32, I32P,
                                         ctypes.POINTER(ctypes.c_float)]),
    "tfhe_gpu_bootstrap_tv": (ctypes.c_int, [VP, VP, VP, VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int,
                                             ctypes.c_int32, VP]),
    "tfhe_client_encrypt_phases": (ctypes.c_int, [ctypes.c_void_p, I32P, ctypes.c_int32, I32P, I32P]),
    "tfhe_client_test_vector": (ctypes.c_int, [ctypes.c_int32, I32P, ctypes.c_int32, I32P]),
    "tfhe_gpu_gate_keyset": (ctypes.c_int, [VP, I32P, I32P, I32P, I32P, ctypes.c_uint32]),
    "tfhe_gpu_selftest_timeout": (ctypes.c_int, [VP, ctypes.c_int, ctypes.c_int32]),
    "tfhe_gpu_measure_fp32_peak": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double)]),
    "tfhe_gpu_measure_fp64_peak": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32,
                                                  ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double)]),
    "tfhe_client_set_seed": (None, [U32P, ctypes.c_int32]),
    "tfhe_client_gate_keyset": (ctypes.c_int, [ctypes.c_void_p, I32P, I32P, I32P, I32P]),
    "tfhe_client_encrypt_bits": (ctypes.c_int, [ctypes.c_void_p, I32P, ctypes.c_int32, I32P, I32P]),
    "tfhe_client_decrypt_bits": (ctypes.c_int, [ctypes.c_void_p, I32P, ctypes.c_int32, I32P, I32P]),
    "tfhe_client_phases": (None, [I32P, ctypes.c_int32, ctypes.c_int32, I32P, I32P]),
    "tfhe_client_mod_switch_to_torus32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
}

_LIB = None


def lib():
    """Load the engine's shared library (fails loudly if it was not built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libtfhe_gb300.so not built: run __graft_entry__.build() "
                              "(nvcc, sm_103a); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _np(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _ptr(x):
    """Device address of a tensor-like object, a raw int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


# ---- client side (host only) -------------------------------------------------

def set_seed(values):
    v = _np(values, np.uint32)
    lib().tfhe_client_set_seed(v.ctypes.data_as(U32P), len(v))


def gate_keyset(P, seed):
    """Seed the generator and produce (lwe_key, tlwe_key, ks, bk) like the
    upstream new_random_gate_bootstrapping_secret_keyset."""
    set_seed(seed)
    lwe = np.zeros(P.n, np.int32)
    tlwe = np.zeros(P.k * P.N, np.int32)
    ks = np.zeros(P.ks_words(), np.int32)
    bk = np.zeros(P.n * P.tgsw_words(), np.int32)
    st = lib().tfhe_client_gate_keyset(ctypes.byref(P), lwe.ctypes.data_as(I32P),
                                       tlwe.ctypes.data_as(I32P), ks.ctypes.data_as(I32P),
                                       bk.ctypes.data_as(I32P))
    if st:
        raise TfheError(st, "gate_keyset")
    return lwe, tlwe, ks, bk


def encrypt_bits(P, bits, lwe_key):
    bits = _np(bits, np.int32)
    out = np.zeros((len(bits), P.n + 1), np.int32)
    st = lib().tfhe_client_encrypt_bits(ctypes.byref(P), bits.ctypes.data_as(I32P), len(bits),
                                        _np(lwe_key, np.int32).ctypes.data_as(I32P),
                                        out.ctypes.data_as(I32P))
    if st:
        raise TfheError(st, "encrypt_bits")
    return out


def encrypt_phases(P, mu, lwe_key):
    """Encrypt Torus32 messages (one per sample)."""
    mu = _np(mu, np.int32)
    out = np.zeros((len(mu), P.n + 1), np.int32)
    st = lib().tfhe_client_encrypt_phases(ctypes.byref(P), mu.ctypes.data_as(I32P), len(mu),
                                          _np(lwe_key, np.int32).ctypes.data_as(I32P),
                                          out.ctypes.data_as(I32P))
    if st:
        raise TfheError(st, "encrypt_phases")
    return out


def test_vector(N, table):
    """Test vector (N int32) of a lookup table on len(table) padded messages."""
    table = _np(table, np.int32)
    tv = np.zeros(N, np.int32)
    st = lib().tfhe_client_test_vector(N, table.ctypes.data_as(I32P), len(table), tv.ctypes.data_as(I32P))
    if st:
        raise TfheError(st, "test_vector")
    return tv


def mod_switch_to_torus32(mu, msize):
    return lib().tfhe_client_mod_switch_to_torus32(int(mu), int(msize))


def decrypt_bits(P, samples, lwe_key):
    s = _np(samples, np.int32).reshape(-1, P.n + 1)
    out = np.zeros(len(s), np.int32)
    st = lib().tfhe_client_decrypt_bits(ctypes.byref(P), s.ctypes.data_as(I32P), len(s),
                                        _np(lwe_key, np.int32).ctypes.data_as(I32P),
                                        out.ctypes.data_as(I32P))
    if st:
        raise TfheError(st, "decrypt_bits")
    return out


def phases(samples, key):
    key = _np(key, np.int32)
    dim = len(key)
    s = _np(samples, np.int32).reshape(-1, dim + 1)
    out = np.zeros(len(s), np.int32)
    lib().tfhe_client_phases(s.ctypes.data_as(I32P), len(s), dim, key.ctypes.data_as(I32P),
                             out.ctypes.data_as(I32P))
    return out


# ---- key and ciphertext files (include/tfhe_keyfile.h) -----------------------

KEYFILE_PARAMS, KEYFILE_CLOUD_KEY, KEYFILE_SECRET_KEY, KEYFILE_CIPHERTEXTS = 1, 2, 3, 4


class _CFile:
    """A C stdio stream on `path` for the FILE*-taking entry points."""
    _libc = None

    def __init__(self, path, mode):
        if _CFile._libc is None:
            libc = ctypes.CDLL(None)
            libc.fopen.restype = VP
            libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
            libc.fclose.restype = ctypes.c_int
            libc.fclose.argtypes = [VP]
            _CFile._libc = libc
        self.f = _CFile._libc.fopen(os.fsencode(path), mode.encode())
        if not self.f:
            raise OSError("cannot open %s" % path)

    def __enter__(self):
        return self.f

    def __exit__(self, *exc):
        if _CFile._libc.fclose(self.f) != 0 and exc[0] is None:
            raise OSError("close failed")


def _kf(st, what):
    if st:
        raise TfheError(st, what)


def keyfile_records(path):
    """[(kind, params)] of every record in a file, in order (headers only)."""
    out = []
    with _CFile(path, "rb") as f:
        L = lib()
        while True:
            kind = ctypes.c_int32()
            P = Params()
            if L.tfhe_keyfile_peek(f, ctypes.byref(kind), ctypes.byref(P), None):
                break
            out.append((kind.value, P))
            # consume the record by reading it (checks the checksum too)
            if kind.value == KEYFILE_PARAMS:
                _kf(L.tfhe_keyfile_read_params(f, None), "read_params")
            elif kind.value == KEYFILE_CLOUD_KEY:
                _kf(L.tfhe_keyfile_read_cloud_key(f, None, None, None), "read_cloud_key")
            elif kind.value == KEYFILE_SECRET_KEY:
                _kf(L.tfhe_keyfile_read_secret_key(f, None, None, None, None, None), "read_secret_key")
            elif kind.value == KEYFILE_CIPHERTEXTS:
                c = ctypes.c_int64(0)
                _kf(L.tfhe_keyfile_read_ciphertexts(f, None, None, None, ctypes.byref(c)),
                    "read_ciphertexts")
            else:
                break
    return out


def save_cloud_key(path, P, bk, ks):
    _kf(lib().tfhe_keyfile_save_cloud_key(os.fsencode(path), ctypes.byref(P),
                                          _np(bk, np.int32).ctypes.data_as(I32P),
                                          _np(ks, np.int32).ctypes.data_as(I32P)), "save_cloud_key")


def load_cloud_key(path):
    """(params, bk, ks) of a cloud-key file."""
    with _CFile(path, "rb") as f:
        kind = ctypes.c_int32()
        P = Params()
        _kf(lib().tfhe_keyfile_peek(f, ctypes.byref(kind), ctypes.byref(P), None), "peek")
    bk = np.zeros(lib().tfhe_keyfile_bk_words(ctypes.byref(P)), np.int32)
    ks = np.zeros(lib().tfhe_keyfile_ks_words(ctypes.byref(P)), np.int32)
    _kf(lib().tfhe_keyfile_load_cloud_key(os.fsencode(path), ctypes.byref(P), bk.ctypes.data_as(I32P),
                                          ks.ctypes.data_as(I32P)), "load_cloud_key")
    return P, bk, ks


def save_secret_key(path, P, lwe_key, tlwe_key, bk, ks):
    with _CFile(path, "wb") as f:
        _kf(lib().tfhe_keyfile_write_secret_key(
            f, ctypes.byref(P), _np(lwe_key, np.int32).ctypes.data_as(I32P),
            _np(tlwe_key, np.int32).ctypes.data_as(I32P), _np(bk, np.int32).ctypes.data_as(I32P),
            _np(ks, np.int32).ctypes.data_as(I32P)), "write_secret_key")


def load_secret_key(path):
    """(params, lwe_key, tlwe_key, bk, ks) of a secret-key file."""
    with _CFile(path, "rb") as f:
        kind = ctypes.c_int32()
        P = Params()
        _kf(lib().tfhe_keyfile_peek(f, ctypes.byref(kind), ctypes.byref(P), None), "peek")
        lwe = np.zeros(P.n, np.int32)
        tlwe = np.zeros(P.k * P.N, np.int32)
        bk = np.zeros(lib().tfhe_keyfile_bk_words(ctypes.byref(P)), np.int32)
        ks = np.zeros(lib().tfhe_keyfile_ks_words(ctypes.byref(P)), np.int32)
        _kf(lib().tfhe_keyfile_read_secret_key(f, ctypes.byref(P), lwe.ctypes.data_as(I32P),
                                               tlwe.ctypes.data_as(I32P), bk.ctypes.data_as(I32P),
                                               ks.ctypes.data_as(I32P)), "read_secret_key")
    return P, lwe, tlwe, bk, ks


def save_ciphertexts(path, P, samples, append=False):
    s = _np(samples, np.int32).reshape(-1, P.n + 1)
    with _CFile(path, "ab" if append else "wb") as f:
        _kf(lib().tfhe_keyfile_write_ciphertexts(f, ctypes.byref(P), s.ctypes.data_as(I32P), None,
                                                 len(s)), "write_ciphertexts")


def load_ciphertexts(path):
    """All ciphertext records of a file, concatenated: int32[count][n+1]."""
    out = []
    with _CFile(path, "rb") as f:
        L = lib()
        while True:
            kind = ctypes.c_int32()
            P = Params()
            items = ctypes.c_int64(0)
            if L.tfhe_keyfile_peek(f, ctypes.byref(kind), ctypes.byref(P), ctypes.byref(items)):
                break
            buf = np.zeros((items.value, P.n + 1), np.int32)
            _kf(L.tfhe_keyfile_read_ciphertexts(f, None, buf.ctypes.data_as(I32P), None,
                                                ctypes.byref(items)), "read_ciphertexts")
            out.append(buf)
    if not out:
        raise TfheError(1, "no ciphertext records in %s" % path)
    return np.concatenate(out)


# ---- engine ------------------------------------------------------------------

class Graph:
    """tfhe_gpu_graph: a captured gate batch, replayed by launch()."""

    def __init__(self, eng, gates, out, ca, cb, count, form, uniform_gate):
        self.eng = eng
        self.lib = eng.lib
        h = VP()
        eng._check(self.lib.tfhe_gpu_graph_gates_create(eng.ctx, _ptr(gates), int(uniform_gate), _ptr(out),
                                                        _ptr(ca), _ptr(cb), int(count), eng._form(form),
                                                        ctypes.byref(h)), "graph_gates_create")
        self.h = h

    @property
    def kernels(self):
        return self.lib.tfhe_gpu_graph_kernel_count(self.h)

    def launch(self, stream=None):
        self.eng._check(self.lib.tfhe_gpu_graph_launch(self.h, stream), "graph_launch")

    def close(self):
        if getattr(self, "h", None):
            self.lib.tfhe_gpu_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One engine context on one device (tfhe_gpu_ctx)."""

    def __init__(self, params=None, device=0):
        self.lib = lib()
        if params is None:
            params = default_params()
        h = VP()
        st = self.lib.tfhe_gpu_create(ctypes.byref(params), int(device), ctypes.byref(h))
        if st:
            raise TfheError(st, "tfhe_gpu_create")
        self.ctx = h
        self.params = Params()
        self.lib.tfhe_gpu_get_params(self.ctx, ctypes.byref(self.params))

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.tfhe_gpu_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st:
            raise TfheError(st, "%s: %s" % (what, self.lib.tfhe_gpu_last_error(self.ctx).decode()))

    @staticmethod
    def _form(form):
        return FORMS[form] if isinstance(form, str) else int(form)

    @property
    def stream(self):
        return self.lib.tfhe_gpu_stream(self.ctx)

    def synchronize(self):
        self._check(self.lib.tfhe_gpu_synchronize(self.ctx), "synchronize")

    def tgsw_fft_bytes(self, form):
        return self.lib.tfhe_gpu_tgsw_fft_bytes(self.ctx, self._form(form))

    def device_bytes(self):
        return self.lib.tfhe_gpu_device_bytes(self.ctx)

    def set_groups_per_cta(self, form, groups):
        """Launch shape of the blind rotation (tfhe_gpu_set_groups_per_cta).
        split_fp32: 0 automatic; 1, 2, 4 L2-direct; 5-8 shared key ring, one
        transform at a time; 9 ring, 4 per CTA, a step's transforms
        together; 10 ring, 6 per CTA, two at a time; 11-13 pair kernel;
        14 spread kernel; 15 automatic in fixed summation order (no pair
        kernel: results independent of the batch); 16 spread kernel over a
        two-SM cluster (lowest latency).  fp64: 0 automatic (the two-SM
        cluster kernel up to one ciphertext per SM, else 3); 3
        L2-direct, 3 per CTA; 4 shared key ring; 16 two-SM cluster."""
        self._check(self.lib.tfhe_gpu_set_groups_per_cta(self.ctx, self._form(form), int(groups)),
                    "set_groups_per_cta")

    def get_groups_per_cta(self, form):
        return self.lib.tfhe_gpu_get_groups_per_cta(self.ctx, self._form(form))

    # keys
    def upload_bootstrapping_key(self, bk, forms=("fp64", "split_fp32")):
        mask = 0
        for f in forms:
            mask |= 1 << self._form(f)
        bk = _np(bk, np.int32)
        self._check(self.lib.tfhe_gpu_upload_bootstrapping_key(self.ctx, bk.ctypes.data_as(I32P), mask),
                    "upload_bootstrapping_key")

    def upload_bootstrapping_key_fft(self, bk_fft, forms=("fp64", "split_fp32")):
        mask = 0
        for f in forms:
            mask |= 1 << self._form(f)
        bk_fft = _np(bk_fft, np.float64)
        self._check(self.lib.tfhe_gpu_upload_bootstrapping_key_fft(
            self.ctx, bk_fft.ctypes.data_as(F64P), mask), "upload_bootstrapping_key_fft")

    def gate_keyset(self, seed, forms=("fp64", "split_fp32"), want_bk=True):
        """Seed the client generator and generate (lwe, tlwe, ks, bk) with the
        bootstrapping key's arithmetic on the GPU; the keys are uploaded."""
        P = self.params
        set_seed(seed)
        lwe = np.zeros(P.n, np.int32)
        tlwe = np.zeros(P.k * P.N, np.int32)
        ks = np.zeros(P.ks_words(), np.int32)
        bk = np.zeros(P.n * P.tgsw_words(), np.int32) if want_bk else None
        mask = 0
        for f in forms:
            mask |= 1 << FORMS[f]
        self._check(self.lib.tfhe_gpu_gate_keyset(self.ctx, lwe.ctypes.data_as(I32P), tlwe.ctypes.data_as(I32P),
                                                  ks.ctypes.data_as(I32P),
                                                  bk.ctypes.data_as(I32P) if want_bk else None, mask),
                    "gate_keyset")
        return lwe, tlwe, ks, bk

    def selftest_timeout(self, form, count):
        """Status of a blind rotation whose key stream never starts (the
        bounded waits run out): 3 = TFHE_GPU_TIMEOUT, 0 for shapes without
        waits."""
        return self.lib.tfhe_gpu_selftest_timeout(self.ctx, self._form(form), int(count))

    def autotune(self, form, count):
        """Time the launch shapes on `count` ciphertexts; keeps and returns
        (shape, ms) of the fastest (the automatic shape unless another is
        more than 2 % faster)."""
        shape = ctypes.c_int32()
        ms = ctypes.c_float()
        self._check(self.lib.tfhe_gpu_autotune(self.ctx, self._form(form), int(count), ctypes.byref(shape),
                                               ctypes.byref(ms)), "autotune")
        return shape.value, ms.value

    def graph_gates(self, gates, out, ca, cb, count, form="split_fp32", uniform_gate=0):
        """A CUDA graph of the gate pipeline over fixed device buffers."""
        return Graph(self, gates, out, ca, cb, count, form, uniform_gate)

    def upload_cloud_key(self, bk, ks, forms=("fp64", "split_fp32")):
        mask = 0
        for f in forms:
            mask |= 1 << FORMS[f]
        self._check(self.lib.tfhe_gpu_upload_cloud_key(self.ctx, _np(bk, np.int32).ctypes.data_as(I32P),
                                                       _np(ks, np.int32).ctypes.data_as(I32P), mask),
                    "upload_cloud_key")

    def upload_cloud_key_file(self, path, forms=("fp64", "split_fp32")):
        mask = 0
        for f in forms:
            mask |= 1 << FORMS[f]
        self._check(self.lib.tfhe_gpu_upload_cloud_key_file(self.ctx, os.fsencode(path), mask),
                    "upload_cloud_key_file")

    def bootsMUX_host(self, a, b, c, form="split_fp32"):
        a, b, c = (_np(x, np.int32).reshape(-1, self.params.n + 1) for x in (a, b, c))
        out = np.zeros_like(a)
        self._check(self.lib.tfhe_gpu_bootsMUX_host(self.ctx, out.ctypes.data_as(I32P),
                                                    a.ctypes.data_as(I32P), b.ctypes.data_as(I32P),
                                                    c.ctypes.data_as(I32P), len(a), self._form(form)),
                    "bootsMUX_host")
        return out

    def upload_keyswitch_key(self, ks):
        ks = _np(ks, np.int32)
        self._check(self.lib.tfhe_gpu_upload_keyswitch_key(self.ctx, ks.ctypes.data_as(I32P)),
                    "upload_keyswitch_key")

    # device-batch entry points (arguments: device buffers)
    def tgsw_to_fft(self, tgsw, out, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_tgsw_to_fft(self.ctx, _ptr(tgsw), _ptr(out), count,
                                                  self._form(form), stream), "tgsw_to_fft")

    def IntPolynomial_ifft(self, polys, out, count, stream=None):
        self._check(self.lib.tfhe_gpu_IntPolynomial_ifft(self.ctx, _ptr(polys), _ptr(out), count, stream),
                    "IntPolynomial_ifft")

    def TorusPolynomial_ifft(self, polys, out, count, stream=None):
        self._check(self.lib.tfhe_gpu_TorusPolynomial_ifft(self.ctx, _ptr(polys), _ptr(out), count,
                                                           stream), "TorusPolynomial_ifft")

    def TorusPolynomial_fft(self, values, polys, count, stream=None):
        self._check(self.lib.tfhe_gpu_TorusPolynomial_fft(self.ctx, _ptr(values), _ptr(polys), count,
                                                          stream), "TorusPolynomial_fft")

    def LagrangeHalfCPolynomialAddMul(self, accum, a, b, count, stream=None):
        self._check(self.lib.tfhe_gpu_LagrangeHalfCPolynomialAddMul(self.ctx, _ptr(accum), _ptr(a), _ptr(b),
                                                                    count, stream),
                    "LagrangeHalfCPolynomialAddMul")

    def tLweMulByXaiMinusOne(self, out, ai, inp, count, stream=None):
        self._check(self.lib.tfhe_gpu_tLweMulByXaiMinusOne(self.ctx, _ptr(out), _ptr(ai), _ptr(inp), count,
                                                           stream), "tLweMulByXaiMinusOne")

    def tGswFFTExternMulToTLwe(self, accum, gsw, count, form, per_item=True, stream=None):
        self._check(self.lib.tfhe_gpu_tGswFFTExternMulToTLwe(self.ctx, _ptr(accum), _ptr(gsw),
                                                             1 if per_item else 0, count,
                                                             self._form(form), stream),
                    "tGswFFTExternMulToTLwe")

    def tfhe_MuxRotate_FFT(self, result, accum, gsw, barai, count, form, per_item=True, stream=None):
        self._check(self.lib.tfhe_gpu_tfhe_MuxRotate_FFT(self.ctx, _ptr(result), _ptr(accum), _ptr(gsw),
                                                         1 if per_item else 0, _ptr(barai), count,
                                                         self._form(form), stream),
                    "tfhe_MuxRotate_FFT")

    def tfhe_blindRotate_FFT(self, accum, bara, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_tfhe_blindRotate_FFT(self.ctx, _ptr(accum), _ptr(bara), count,
                                                           self._form(form), stream),
                    "tfhe_blindRotate_FFT")

    def tLweExtractLweSample(self, out, accum, count, stream=None):
        self._check(self.lib.tfhe_gpu_tLweExtractLweSample(self.ctx, _ptr(out), _ptr(accum), count,
                                                           stream), "tLweExtractLweSample")

    def lweKeySwitch(self, out, inp, count, stream=None):
        self._check(self.lib.tfhe_gpu_lweKeySwitch(self.ctx, _ptr(out), _ptr(inp), count, stream),
                    "lweKeySwitch")

    def tfhe_bootstrap_woKS_FFT(self, out, x, mu, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_tfhe_bootstrap_woKS_FFT(self.ctx, _ptr(out), _ptr(x), int(mu),
                                                              count, self._form(form), stream),
                    "tfhe_bootstrap_woKS_FFT")

    def tfhe_bootstrap_FFT(self, out, x, mu, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_tfhe_bootstrap_FFT(self.ctx, _ptr(out), _ptr(x), int(mu), count,
                                                         self._form(form), stream),
                    "tfhe_bootstrap_FFT")

    def bootsGate(self, gate, out, ca, cb, count, form, stream=None):
        g = GATES[gate] if isinstance(gate, str) else int(gate)
        self._check(self.lib.tfhe_gpu_bootsGate(self.ctx, g, _ptr(out), _ptr(ca), _ptr(cb), count,
                                                self._form(form), stream), "bootsGate")

    def bootstrap_tv(self, out, x, tv, count, form, tv_stride=0, keyswitch=True, stream=None):
        """Programmable bootstrap of `count` samples with test vector(s) tv."""
        self._check(self.lib.tfhe_gpu_bootstrap_tv(self.ctx, _ptr(out), _ptr(x), _ptr(tv), int(tv_stride),
                                                   int(count), self._form(form), 1 if keyswitch else 0,
                                                   stream), "bootstrap_tv")

    def bootsGates(self, gates, out, ca, cb, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_bootsGates(self.ctx, _ptr(gates), _ptr(out), _ptr(ca), _ptr(cb),
                                                 count, self._form(form), stream), "bootsGates")

    def bootsGates_noalloc(self, gates, out, ca, cb, count, form, stream=None):
        """tfhe_gpu_bootsGates without any allocation inside the call (fixed
        device scratch in the library; up to 512 gates of the default set;
        calls overlapping on the GPU must be serialised)."""
        self._check(self.lib.tfhe_gpu_bootsGates_noalloc(self.ctx, _ptr(gates), _ptr(out), _ptr(ca),
                                                         _ptr(cb), count, self._form(form), stream),
                    "bootsGates_noalloc")

    def bootsMUX(self, out, a, b, c, count, form, stream=None):
        self._check(self.lib.tfhe_gpu_bootsMUX(self.ctx, _ptr(out), _ptr(a), _ptr(b), _ptr(c), count,
                                               self._form(form), stream), "bootsMUX")

    # host-buffer form (end to end)
    def bootsGates_host(self, ca, cb, gates=None, gate="NAND", form="split_fp32", out=None):
        ca = _np(ca, np.int32)
        cb = _np(cb, np.int32)
        count = ca.shape[0]
        if out is None:
            out = np.zeros_like(ca)
        gp = None
        if gates is not None:
            gates = _np(gates, np.int32)
            gp = gates.ctypes.data_as(I32P)
        g = GATES[gate] if isinstance(gate, str) else int(gate)
        self._check(self.lib.tfhe_gpu_bootsGates_host(self.ctx, gp, g, out.ctypes.data_as(I32P),
                                                      ca.ctypes.data_as(I32P), cb.ctypes.data_as(I32P),
                                                      count, self._form(form)), "bootsGates_host")
        return out


def bootsGates_host_split(engines, ca, cb, gates=None, gate="NAND", form="split_fp32", out=None):
    """One layer of gates over several engines (tfhe_gpu_bootsGates_host_split):
    contiguous shards, one per engine, run concurrently; outputs in layer
    order.  The engines must be distinct and hold the same keys."""
    ca = _np(ca, np.int32)
    cb = _np(cb, np.int32)
    if out is None:
        out = np.zeros_like(ca)
    gp = None
    if gates is not None:
        gates = _np(gates, np.int32)
        gp = gates.ctypes.data_as(I32P)
    arr = (VP * len(engines))(*[e.ctx for e in engines])
    g = GATES[gate] if isinstance(gate, str) else int(gate)
    st = lib().tfhe_gpu_bootsGates_host_split(arr, len(engines), gp, g, out.ctypes.data_as(I32P),
                                              ca.ctypes.data_as(I32P), cb.ctypes.data_as(I32P), ca.shape[0],
                                              Engine._form(form))
    if st:
        details = "; ".join(lib().tfhe_gpu_last_error(e.ctx).decode() for e in engines)
        raise TfheError(st, "bootsGates_host_split: " + details)
    return out


class Server:
    """Continuous-batching gate server (tfhe_gpu_server_*) over an Engine."""

    def __init__(self, engine, pool_slots=65536, max_batch=4096, form="split_fp32"):
        self.engine = engine
        self.lib = engine.lib
        h = VP()
        st = self.lib.tfhe_gpu_server_create(engine.ctx, int(pool_slots), int(max_batch),
                                             engine._form(form), ctypes.byref(h))
        if st:
            raise TfheError(st, "tfhe_gpu_server_create")
        self.srv = h
        self.width = engine.params.n + 1
        self.noutputs = {}

    def close(self):
        if getattr(self, "srv", None):
            self.lib.tfhe_gpu_server_destroy(self.srv)
            self.srv = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st:
            raise TfheError(st, "%s: %s" % (what, self.lib.tfhe_gpu_server_last_error(self.srv).decode()))

    def submit(self, gates, ninputs, inputs, outputs):
        """gates: int32 [ngates, 4] (type, in0, in1, in2); inputs: int32
        [ninputs, n+1]; outputs: wire ids.  Returns the request id."""
        g = _np(gates, np.int32).reshape(-1, 4)
        x = _np(inputs, np.int32).reshape(-1, self.width)
        o = _np(outputs, np.int32)
        rid = ctypes.c_int64()
        self._check(self.lib.tfhe_gpu_server_submit(self.srv, g.ctypes.data_as(I32P), len(g), int(ninputs),
                                                    x.ctypes.data_as(I32P), o.ctypes.data_as(I32P), len(o),
                                                    ctypes.byref(rid)), "submit")
        self.noutputs[rid.value] = len(o)
        return rid.value

    def step(self):
        ran = ctypes.c_int32()
        self._check(self.lib.tfhe_gpu_server_step(self.srv, ctypes.byref(ran)), "step")
        return ran.value

    def poll(self, rid):
        """(outputs, latency_s) of a finished request, or None."""
        out = np.zeros((self.noutputs[rid], self.width), np.int32)
        done = ctypes.c_int32()
        lat = ctypes.c_double()
        self._check(self.lib.tfhe_gpu_server_poll(self.srv, int(rid), out.ctypes.data_as(I32P),
                                                  ctypes.byref(done), ctypes.byref(lat)), "poll")
        if not done.value:
            return None
        del self.noutputs[rid]
        return out, lat.value

    def stats(self):
        st = np.zeros(8, np.float64)
        cap = (ctypes.c_int64 * 2)(0, 0)
        self._check(self.lib.tfhe_gpu_server_stats(self.srv, st.ctypes.data_as(F64P), None, None, cap),
                    "stats")
        g = np.zeros(max(cap[0], 1), np.float64)
        r = np.zeros(max(cap[1], 1), np.float64)
        self._check(self.lib.tfhe_gpu_server_stats(self.srv, st.ctypes.data_as(F64P), g.ctypes.data_as(F64P),
                                                   r.ctypes.data_as(F64P), cap), "stats")
        keys = ["queued", "active", "free_slots", "bootstraps", "busy_s", "n_gate_lat", "n_req_lat", "pool_slots"]
        d = dict(zip(keys, st.tolist()))
        d["gate_latency_s"] = g[:cap[0]]
        d["request_latency_s"] = r[:cap[1]]
        return d
