"""ctypes loader of oracle/_ref/ (the reference's own CPU-path code built by
build_ref.py).  Test infrastructure only.

The reference's MuxRotate and blind-rotation files open text log files in
the working directory: MuxRotate when the library loads
(tfhe_MuxRotate_FFT.cpp:5-7), the blind rotation on every call
(tfhe_blindRotate_FFT.cpp:85).  The loader switches to a private temporary
directory while loading and around every call into the hot-path library, so
that those files land there and never in the caller's directory.
"""
import contextlib
import ctypes
import functools
import os
import tempfile

import numpy as np

from . import build_ref

I32P = ctypes.POINTER(ctypes.c_int32)
U32P = ctypes.POINTER(ctypes.c_uint32)
F64P = ctypes.POINTER(ctypes.c_double)

_REF = None


def _p(a, t):
    return a.ctypes.data_as(t)


def _in_logdir(method):
    """Run a method that calls into libref_hls.so from the log directory."""
    @functools.wraps(method)
    def wrapped(self, *args, **kwargs):
        with self.logs():
            return method(self, *args, **kwargs)
    return wrapped


class Reference:
    def __init__(self):
        paths = build_ref.build(quiet=True)
        if paths is None:
            raise RuntimeError("reference sources not available on this machine")
        self.logdir = tempfile.mkdtemp(prefix="ref_logs_")
        cwd = os.getcwd()
        os.chdir(self.logdir)
        try:
            self.hls = ctypes.CDLL(paths[0])
            self.tfhe = ctypes.CDLL(paths[1])
        finally:
            os.chdir(cwd)
        H, T = self.hls, self.tfhe
        for name, args in {"refh_decompose": [I32P, I32P], "refh_decomp_h": [I32P, I32P],
                           "refh_int_ifft": [I32P, F64P], "refh_torus_fft": [F64P, I32P],
                           "refh_extern_mul": [I32P, F64P],
                           "refh_mux_rotate": [I32P, I32P, F64P, ctypes.c_int32],
                           "refh_blind_rotate": [I32P, F64P, I32P, ctypes.c_int32],
                           "refh_blind_rotate_shipped": [I32P, F64P, I32P],
                           "refh_bootstrap_front": [I32P, ctypes.c_int32, I32P, I32P, I32P, I32P],
                           "refh_params": [I32P]}.items():
            f = getattr(H, name)
            f.argtypes = args
            f.restype = ctypes.c_int32 if name == "refh_params" else None
        for name, (res, args) in {
                "tfhe_random_generator_setSeed": (None, [U32P, ctypes.c_int32]),
                "gaussian32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_double]),
                "dtot32": (ctypes.c_int32, [ctypes.c_double]),
                "approxPhase": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
                "modSwitchFromTorus32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
                "modSwitchToTorus32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
                "refu_lwe_keygen": (None, [ctypes.c_int32, I32P]),
                "refu_lwe_encrypt": (None, [ctypes.c_int32, I32P, ctypes.c_int32, ctypes.c_double, I32P]),
                "refu_lwe_phase": (ctypes.c_int32, [ctypes.c_int32, I32P, I32P]),
                "refu_create_ks_key": (None, [ctypes.c_int32, I32P, ctypes.c_int32, I32P, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_double, I32P]),
                "refu_keyswitch": (None, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          I32P, I32P, I32P]),
                "refu_or_combination": (None, [ctypes.c_int32, ctypes.c_int32, I32P, I32P, I32P])}.items():
            f = getattr(T, name)
            f.restype = res
            f.argtypes = args
        pv = np.zeros(7, np.int32)
        H.refh_params(_p(pv, I32P))
        self.n, self.N, self.k, self.l, self.Bgbit, self.ks_t, self.ks_basebit = (int(x) for x in pv)

    @contextlib.contextmanager
    def logs(self):
        """Working directory = the private log directory for the duration."""
        cwd = os.getcwd()
        os.chdir(self.logdir)
        try:
            yield
        finally:
            os.chdir(cwd)

    # numeric / LWE (numeric-functions.cpp, lwe-functions.cpp)
    def set_seed(self, values):
        v = np.ascontiguousarray(values, np.uint32)
        self.tfhe.tfhe_random_generator_setSeed(_p(v, U32P), len(v))

    def lwe_keygen(self, n):
        out = np.zeros(n, np.int32)
        self.tfhe.refu_lwe_keygen(n, _p(out, I32P))
        return out

    def lwe_encrypt(self, key, message, alpha):
        key = np.ascontiguousarray(key, np.int32)
        out = np.zeros(len(key) + 1, np.int32)
        self.tfhe.refu_lwe_encrypt(len(key), _p(key, I32P), int(message), alpha, _p(out, I32P))
        return out

    def create_ks_key(self, in_key, out_key, t, basebit, alpha):
        in_key = np.ascontiguousarray(in_key, np.int32)
        out_key = np.ascontiguousarray(out_key, np.int32)
        out = np.zeros(len(in_key) * t * (1 << basebit) * (len(out_key) + 1), np.int32)
        self.tfhe.refu_create_ks_key(len(in_key), _p(in_key, I32P), len(out_key), _p(out_key, I32P), t,
                                     basebit, alpha, _p(out, I32P))
        return out

    def keyswitch(self, table, sample, n_in, n_out, t, basebit):
        out = np.zeros(n_out + 1, np.int32)
        self.tfhe.refu_keyswitch(n_in, n_out, t, basebit, _p(np.ascontiguousarray(table, np.int32), I32P),
                                 _p(np.ascontiguousarray(sample, np.int32), I32P), _p(out, I32P))
        return out

    def or_combination(self, c, ca, cb):
        n = len(ca) - 1
        out = np.zeros(n + 1, np.int32)
        self.tfhe.refu_or_combination(n, int(c), _p(np.ascontiguousarray(ca, np.int32), I32P),
                                      _p(np.ascontiguousarray(cb, np.int32), I32P), _p(out, I32P))
        return out

    # hot-path kernels (tfhe_blindRotate_FFT/*.cpp)
    @_in_logdir
    def decompose(self, poly):
        out = np.zeros(self.l * self.N, np.int32)
        self.hls.refh_decompose(_p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, I32P))
        return out.reshape(self.l, self.N)

    @_in_logdir
    def decomp_h(self, poly):
        out = np.zeros(self.l * self.N, np.int32)
        self.hls.refh_decomp_h(_p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, I32P))
        return out.reshape(self.l, self.N)

    @_in_logdir
    def int_ifft(self, poly):
        out = np.zeros(self.N, np.float64)
        self.hls.refh_int_ifft(_p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, F64P))
        return out[0::2] + 1j * out[1::2]

    @_in_logdir
    def torus_fft(self, values):
        v = np.ascontiguousarray(np.stack([np.real(values), np.imag(values)], -1).reshape(-1), np.float64)
        out = np.zeros(self.N, np.int32)
        self.hls.refh_torus_fft(_p(v, F64P), _p(out, I32P))
        return out

    @_in_logdir
    def extern_mul(self, accum, gsw_fft):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.hls.refh_extern_mul(_p(acc, I32P), _p(np.ascontiguousarray(gsw_fft, np.float64), F64P))
        return acc

    @_in_logdir
    def mux_rotate(self, accum, bki_fft, barai):
        out = np.zeros((self.k + 1) * self.N, np.int32)
        self.hls.refh_mux_rotate(_p(out, I32P), _p(np.ascontiguousarray(accum, np.int32), I32P),
                                 _p(np.ascontiguousarray(bki_fft, np.float64), F64P), int(barai))
        return out

    @_in_logdir
    def blind_rotate(self, accum, bk_fft, bara):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        bara = np.ascontiguousarray(bara, np.int32)
        self.hls.refh_blind_rotate(_p(acc, I32P), _p(np.ascontiguousarray(bk_fft, np.float64), F64P),
                                   _p(bara, I32P), len(bara))
        return acc

    @_in_logdir
    def blind_rotate_shipped(self, accum, bk0_fft, bara):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.hls.refh_blind_rotate_shipped(_p(acc, I32P), _p(np.ascontiguousarray(bk0_fft, np.float64), F64P),
                                           _p(np.ascontiguousarray(bara, np.int32), I32P))
        return acc

    @_in_logdir
    def bootstrap_front(self, x, mu):
        tv = np.zeros(self.N, np.int32)
        bara = np.zeros(self.n, np.int32)
        barb = np.zeros(1, np.int32)
        rot = np.zeros(self.N, np.int32)
        self.hls.refh_bootstrap_front(_p(np.ascontiguousarray(x, np.int32), I32P), int(mu), _p(tv, I32P),
                                      _p(bara, I32P), _p(barb, I32P), _p(rot, I32P))
        return tv, bara, int(barb[0]), rot


def available():
    return build_ref.available()


def get():
    global _REF
    if _REF is None:
        _REF = Reference()
    return _REF
