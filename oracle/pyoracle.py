"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by tests/, by __graft_entry__.smoke() to check its result, and by the
cpu_baseline / reference leg of bench.py.  The engine never imports this.
"""
import ctypes
import os

import numpy as np

from . import build_oracle  # noqa: F401  (package-relative when imported as oracle.pyoracle)

I32P = ctypes.POINTER(ctypes.c_int32)
U32P = ctypes.POINTER(ctypes.c_uint32)
F64P = ctypes.POINTER(ctypes.c_double)


class Params(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("N", ctypes.c_int32), ("k", ctypes.c_int32),
                ("l", ctypes.c_int32), ("Bgbit", ctypes.c_int32), ("ks_t", ctypes.c_int32),
                ("ks_basebit", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("lwe_alpha", ctypes.c_double), ("tlwe_alpha", ctypes.c_double)]

    @property
    def kpl(self):
        return (self.k + 1) * self.l

    def tgsw_words(self):
        return self.kpl * (self.k + 1) * self.N

    def ks_words(self):
        return self.k * self.N * self.ks_t * (1 << self.ks_basebit) * (self.n + 1)


def default_params():
    """The 110-bit default gate set (constants.h:26-40)."""
    return Params(n=630, N=1024, k=1, l=3, Bgbit=7, ks_t=8, ks_basebit=2, pad_=0,
                  lwe_alpha=2.0 ** -15, tlwe_alpha=2.0 ** -25)


def stress_params():
    """Alternative set n=500, l=2, Bgbit=10, LWE 2^-15, TRLWE 2^-24."""
    return Params(n=500, N=1024, k=1, l=2, Bgbit=10, ks_t=8, ks_basebit=2, pad_=0,
                  lwe_alpha=2.0 ** -15, tlwe_alpha=2.0 ** -24)


GATES = {"NAND": 0, "AND": 1, "OR": 2, "XOR": 3, "XNOR": 4, "NOR": 5,
         "ANDNY": 6, "ANDYN": 7, "ORNY": 8, "ORYN": 9}

GATE_FN = {
    "NAND": lambda a, b: 1 - (a & b), "AND": lambda a, b: a & b,
    "OR": lambda a, b: a | b, "XOR": lambda a, b: a ^ b,
    "XNOR": lambda a, b: 1 - (a ^ b), "NOR": lambda a, b: 1 - (a | b),
    "ANDNY": lambda a, b: (1 - a) & b, "ANDYN": lambda a, b: a & (1 - b),
    "ORNY": lambda a, b: (1 - a) | b, "ORYN": lambda a, b: a | (1 - b),
}


def _p(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    def __init__(self, lib_path=None):
        if lib_path is None:
            lib_path = build_oracle.build()
        self.lib = ctypes.CDLL(lib_path)
        L = self.lib
        PP = ctypes.POINTER(Params)
        sig = {
            "orc_set_seed": (None, [U32P, ctypes.c_int32]),
            "orc_uniform_torus32": (ctypes.c_int32, []),
            "orc_gaussian32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_double]),
            "orc_dtot32": (ctypes.c_int32, [ctypes.c_double]),
            "orc_mod_switch_from_torus32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
            "orc_mod_switch_to_torus32": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
            "orc_approx_phase": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
            "orc_lwe_keygen": (None, [I32P, ctypes.c_int32]),
            "orc_lwe_encrypt": (None, [I32P, ctypes.c_int32, ctypes.c_double, I32P, ctypes.c_int32]),
            "orc_lwe_phase": (ctypes.c_int32, [I32P, I32P, ctypes.c_int32]),
            "orc_tlwe_keygen": (None, [I32P, ctypes.c_int32, ctypes.c_int32]),
            "orc_tgsw_encrypt_int": (None, [PP, I32P, ctypes.c_int32, ctypes.c_double, I32P]),
            "orc_create_ks_key": (None, [PP, I32P, I32P, ctypes.c_int32, I32P]),
            "orc_gate_keyset": (None, [PP, I32P, I32P, I32P, I32P]),
            "orc_boots_sym_encrypt": (None, [PP, I32P, ctypes.c_int32, I32P]),
            "orc_boots_sym_decrypt": (ctypes.c_int32, [PP, I32P, I32P]),
            "orc_decompose": (None, [PP, I32P, I32P]),
            "orc_int_poly_ifft": (None, [ctypes.c_int32, I32P, F64P]),
            "orc_torus_poly_ifft": (None, [ctypes.c_int32, I32P, F64P]),
            "orc_torus_poly_fft": (None, [ctypes.c_int32, F64P, I32P]),
            "orc_tgsw_to_fft": (None, [PP, I32P, F64P]),
            "orc_bk_to_fft": (None, [PP, I32P, F64P]),
            "orc_mul_by_xai": (None, [ctypes.c_int32, ctypes.c_int32, I32P, I32P]),
            "orc_mul_by_xai_minus_one": (None, [ctypes.c_int32, ctypes.c_int32, I32P, I32P]),
            "orc_extern_mul_fft": (None, [PP, I32P, F64P]),
            "orc_extern_mul_exact": (None, [PP, I32P, I32P]),
            "orc_mux_rotate_fft": (None, [PP, I32P, I32P, F64P, ctypes.c_int32]),
            "orc_blind_rotate_fft": (None, [PP, I32P, F64P, I32P]),
            "orc_blind_rotate_exact": (None, [PP, I32P, I32P, I32P]),
            "orc_extract": (None, [PP, I32P, I32P]),
            "orc_keyswitch": (None, [PP, I32P, I32P, I32P]),
            "orc_bootstrap_prologue": (None, [PP, ctypes.c_int32, I32P, I32P, I32P]),
            "orc_bootstrap_woks": (None, [PP, F64P, ctypes.c_int32, I32P, I32P, ctypes.c_int32, I32P]),
            "orc_gate_combine": (None, [PP, ctypes.c_int32, I32P, I32P, I32P]),
            "orc_boots_gate": (None, [PP, F64P, I32P, ctypes.c_int32, I32P, I32P, I32P]),
            "orc_boots_mux": (None, [PP, F64P, I32P, I32P, I32P, I32P, I32P]),
            "orc_boots_mux_batch": (None, [PP, F64P, I32P, I32P, I32P, I32P, I32P, ctypes.c_int32,
                                           ctypes.c_int32]),
            "orc_boots_gate_batch": (None, [PP, F64P, I32P, I32P, I32P, I32P, I32P,
                                            ctypes.c_int32, ctypes.c_int32]),
            "orc_extern_mul_exact_batch": (None, [PP, I32P, I32P, ctypes.c_int32, ctypes.c_int32]),
            "orc_bootstrap_woks_batch": (None, [PP, F64P, ctypes.c_int32, I32P, I32P, ctypes.c_int32,
                                                ctypes.c_int32, I32P, ctypes.c_int32]),
            "orc_boots_gate_exact_batch": (None, [PP, I32P, I32P, I32P, I32P, I32P, I32P,
                                                  ctypes.c_int32, ctypes.c_int32]),
            "orc_max_threads": (ctypes.c_int32, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args

    # -- scalar helpers ------------------------------------------------
    def set_seed(self, values):
        v = np.ascontiguousarray(np.asarray(values, dtype=np.uint32))
        self.lib.orc_set_seed(_p(v, U32P), len(v))

    def __getattr__(self, name):
        # direct access to scalar functions: o.mod_switch_to_torus32(1, 8)
        f = getattr(self.lib, "orc_" + name)
        return f

    # -- keys ----------------------------------------------------------
    def gate_keyset(self, P, seed):
        """Generate (lwe_key, tlwe_key, ks, bk) the way the upstream
        new_random_gate_bootstrapping_secret_keyset does, after seeding."""
        self.set_seed(seed)
        lwe_key = np.zeros(P.n, np.int32)
        tlwe_key = np.zeros(P.k * P.N, np.int32)
        ks = np.zeros(P.ks_words(), np.int32)
        bk = np.zeros(P.n * P.tgsw_words(), np.int32)
        self.lib.orc_gate_keyset(ctypes.byref(P), _p(lwe_key, I32P), _p(tlwe_key, I32P),
                                 _p(ks, I32P), _p(bk, I32P))
        return lwe_key, tlwe_key, ks, bk

    def bk_to_fft(self, P, bk):
        out = np.zeros(P.n * P.tgsw_words(), np.float64)
        self.lib.orc_bk_to_fft(ctypes.byref(P), _p(np.ascontiguousarray(bk), I32P), _p(out, F64P))
        return out

    def tgsw_encrypt_int(self, P, message, alpha, tlwe_key):
        out = np.zeros(P.tgsw_words(), np.int32)
        self.lib.orc_tgsw_encrypt_int(ctypes.byref(P), _p(out, I32P), int(message), alpha,
                                      _p(np.ascontiguousarray(tlwe_key, np.int32), I32P))
        return out

    def tgsw_to_fft(self, P, tgsw):
        out = np.zeros(P.tgsw_words(), np.float64)
        self.lib.orc_tgsw_to_fft(ctypes.byref(P), _p(np.ascontiguousarray(tgsw, np.int32), I32P),
                                 _p(out, F64P))
        return out

    # -- LWE -----------------------------------------------------------
    def encrypt_bits(self, P, bits, lwe_key):
        out = np.zeros((len(bits), P.n + 1), np.int32)
        for i, b in enumerate(bits):
            row = out[i]
            self.lib.orc_boots_sym_encrypt(ctypes.byref(P), _p(row, I32P), int(b), _p(lwe_key, I32P))
        return out

    def decrypt_bits(self, P, samples, lwe_key):
        s = np.ascontiguousarray(samples, np.int32).reshape(-1, P.n + 1)
        return np.array([self.lib.orc_boots_sym_decrypt(ctypes.byref(P), _p(np.ascontiguousarray(r), I32P),
                                                        _p(lwe_key, I32P)) for r in s], np.int32)

    def phases(self, samples, key, n):
        s = np.ascontiguousarray(samples, np.int32).reshape(-1, n + 1)
        return np.array([self.lib.orc_lwe_phase(_p(np.ascontiguousarray(r), I32P), _p(key, I32P), n)
                         for r in s], np.int32)

    # -- hot path --------------------------------------------------------
    def decompose(self, P, poly):
        out = np.zeros(P.l * P.N, np.int32)
        self.lib.orc_decompose(ctypes.byref(P), _p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, I32P))
        return out.reshape(P.l, P.N)

    def int_poly_ifft(self, N, poly):
        out = np.zeros(N, np.float64)
        self.lib.orc_int_poly_ifft(N, _p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, F64P))
        return out[0::2] + 1j * out[1::2]

    def torus_poly_ifft(self, N, poly):
        out = np.zeros(N, np.float64)
        self.lib.orc_torus_poly_ifft(N, _p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, F64P))
        return out[0::2] + 1j * out[1::2]

    def torus_poly_fft(self, N, values):
        v = np.ascontiguousarray(np.stack([np.real(values), np.imag(values)], -1).reshape(-1), np.float64)
        out = np.zeros(N, np.int32)
        self.lib.orc_torus_poly_fft(N, _p(v, F64P), _p(out, I32P))
        return out

    def mul_by_xai(self, N, a, poly):
        out = np.zeros(N, np.int32)
        self.lib.orc_mul_by_xai(N, int(a), _p(np.ascontiguousarray(poly, np.int32), I32P), _p(out, I32P))
        return out

    def mul_by_xai_minus_one(self, N, a, poly):
        out = np.zeros(N, np.int32)
        self.lib.orc_mul_by_xai_minus_one(N, int(a), _p(np.ascontiguousarray(poly, np.int32), I32P),
                                          _p(out, I32P))
        return out

    def extern_mul_fft(self, P, accum, gsw_fft):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.lib.orc_extern_mul_fft(ctypes.byref(P), _p(acc, I32P),
                                    _p(np.ascontiguousarray(gsw_fft, np.float64), F64P))
        return acc

    def extern_mul_exact(self, P, accum, gsw):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.lib.orc_extern_mul_exact(ctypes.byref(P), _p(acc, I32P),
                                      _p(np.ascontiguousarray(gsw, np.int32), I32P))
        return acc

    def mux_rotate_fft(self, P, accum, bki_fft, barai):
        out = np.zeros((P.k + 1) * P.N, np.int32)
        self.lib.orc_mux_rotate_fft(ctypes.byref(P), _p(out, I32P),
                                    _p(np.ascontiguousarray(accum, np.int32), I32P),
                                    _p(np.ascontiguousarray(bki_fft, np.float64), F64P), int(barai))
        return out

    def blind_rotate_fft(self, P, accum, bk_fft, bara):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.lib.orc_blind_rotate_fft(ctypes.byref(P), _p(acc, I32P), _p(bk_fft, F64P),
                                      _p(np.ascontiguousarray(bara, np.int32), I32P))
        return acc

    def blind_rotate_exact(self, P, accum, bk, bara):
        acc = np.array(accum, np.int32, copy=True).reshape(-1)
        self.lib.orc_blind_rotate_exact(ctypes.byref(P), _p(acc, I32P), _p(bk, I32P),
                                        _p(np.ascontiguousarray(bara, np.int32), I32P))
        return acc

    def extract(self, P, accum):
        out = np.zeros(P.k * P.N + 1, np.int32)
        self.lib.orc_extract(ctypes.byref(P), _p(np.ascontiguousarray(accum, np.int32), I32P), _p(out, I32P))
        return out

    def keyswitch(self, P, ks, sample):
        out = np.zeros(P.n + 1, np.int32)
        self.lib.orc_keyswitch(ctypes.byref(P), _p(ks, I32P), _p(np.ascontiguousarray(sample, np.int32), I32P),
                               _p(out, I32P))
        return out

    def bootstrap_prologue(self, P, mu, x):
        bara = np.zeros(P.n, np.int32)
        acc = np.zeros((P.k + 1) * P.N, np.int32)
        self.lib.orc_bootstrap_prologue(ctypes.byref(P), int(mu), _p(np.ascontiguousarray(x, np.int32), I32P),
                                        _p(bara, I32P), _p(acc, I32P))
        return bara, acc

    def bootstrap_woks(self, P, bk_fft, mu, x, exact_bk=None):
        out = np.zeros(P.k * P.N + 1, np.int32)
        exact = exact_bk is not None
        bkp = _p(exact_bk, I32P) if exact else None
        bkf = _p(bk_fft, F64P) if bk_fft is not None else None
        self.lib.orc_bootstrap_woks(ctypes.byref(P), bkf, int(mu),
                                    _p(np.ascontiguousarray(x, np.int32), I32P), _p(out, I32P),
                                    1 if exact else 0, bkp)
        return out

    def gate_combine(self, P, gate, ca, cb):
        out = np.zeros(P.n + 1, np.int32)
        self.lib.orc_gate_combine(ctypes.byref(P), GATES[gate] if isinstance(gate, str) else int(gate),
                                  _p(np.ascontiguousarray(ca, np.int32), I32P),
                                  _p(np.ascontiguousarray(cb, np.int32), I32P), _p(out, I32P))
        return out

    def boots_gate(self, P, bk_fft, ks, gate, ca, cb):
        out = np.zeros(P.n + 1, np.int32)
        self.lib.orc_boots_gate(ctypes.byref(P), _p(bk_fft, F64P), _p(ks, I32P),
                                GATES[gate] if isinstance(gate, str) else int(gate),
                                _p(np.ascontiguousarray(ca, np.int32), I32P),
                                _p(np.ascontiguousarray(cb, np.int32), I32P), _p(out, I32P))
        return out

    def boots_mux(self, P, bk_fft, ks, a, b, c):
        out = np.zeros(P.n + 1, np.int32)
        self.lib.orc_boots_mux(ctypes.byref(P), _p(bk_fft, F64P), _p(ks, I32P),
                               _p(np.ascontiguousarray(a, np.int32), I32P),
                               _p(np.ascontiguousarray(b, np.int32), I32P),
                               _p(np.ascontiguousarray(c, np.int32), I32P), _p(out, I32P))
        return out

    def boots_mux_batch(self, P, bk_fft, ks, a, b, c, threads=0):
        """bootsMUX of count triples of samples (each count x (n+1)) on
        `threads` host threads (0: all)."""
        a = np.ascontiguousarray(a, np.int32)
        b = np.ascontiguousarray(b, np.int32)
        c = np.ascontiguousarray(c, np.int32)
        out = np.zeros_like(a)
        self.lib.orc_boots_mux_batch(ctypes.byref(P), _p(bk_fft, F64P), _p(ks, I32P), _p(a, I32P), _p(b, I32P),
                                     _p(c, I32P), _p(out, I32P), len(a), int(threads))
        return out

    def test_vector(self, N, table):
        table = np.ascontiguousarray(table, np.int32)
        tv = np.zeros(N, np.int32)
        self.lib.orc_test_vector(N, _p(table, I32P), len(table), _p(tv, I32P))
        return tv

    def bootstrap_tv_batch(self, P, bk_fft, ks, tv, x, threads=0):
        """Programmable bootstrap + key switch of the samples x (count x
        (n+1)); tv is one vector (N) or one per sample (count x N)."""
        x = np.ascontiguousarray(x, np.int32).reshape(-1, P.n + 1)
        tv = np.ascontiguousarray(tv, np.int32)
        stride = P.N if tv.ndim == 2 else 0
        out = np.zeros_like(x)
        self.lib.orc_bootstrap_tv_batch(ctypes.byref(P), _p(bk_fft, F64P), _p(ks, I32P), _p(tv, I32P),
                                        stride, _p(x, I32P), _p(out, I32P), len(x), int(threads))
        return out

    def boots_gate_batch(self, P, bk_fft, ks, gates, ca, cb, threads=0):
        gates = np.ascontiguousarray(gates, np.int32)
        ca = np.ascontiguousarray(ca, np.int32)
        cb = np.ascontiguousarray(cb, np.int32)
        out = np.zeros_like(ca)
        self.lib.orc_boots_gate_batch(ctypes.byref(P), _p(bk_fft, F64P), _p(ks, I32P), _p(gates, I32P),
                                      _p(ca, I32P), _p(cb, I32P), _p(out, I32P), len(gates), int(threads))
        return out


    def extern_mul_exact_batch(self, P, accum, gsw, threads=0):
        """Exact int64 external products of count TRLWE samples (count x
        (k+1)N) by count time-domain TGSW samples."""
        acc = np.array(accum, np.int32, copy=True).reshape(-1, (P.k + 1) * P.N)
        gsw = np.ascontiguousarray(gsw, np.int32).reshape(len(acc), -1)
        self.lib.orc_extern_mul_exact_batch(ctypes.byref(P), _p(acc, I32P), _p(gsw, I32P), len(acc),
                                            int(threads))
        return acc

    def bootstrap_woks_batch(self, P, bk_fft, mu, x, exact_bk=None, threads=0):
        """Bootstraps without key switch of the samples x (count x (n+1)):
        the FFT blind rotation, or the exact int64 one when exact_bk (the
        time-domain key) is given."""
        x = np.ascontiguousarray(x, np.int32).reshape(-1, P.n + 1)
        out = np.zeros((len(x), P.k * P.N + 1), np.int32)
        exact = exact_bk is not None
        self.lib.orc_bootstrap_woks_batch(
            ctypes.byref(P), _p(bk_fft, F64P) if bk_fft is not None else None, int(mu), _p(x, I32P),
            _p(out, I32P), len(x), 1 if exact else 0,
            _p(np.ascontiguousarray(exact_bk, np.int32), I32P) if exact else None, int(threads))
        return out

    def boots_gate_exact_batch(self, P, bk, ks, gates, ca, cb, threads=0):
        """Gates through the exact int64 blind rotation (bk: time-domain key)."""
        gates = np.ascontiguousarray(gates, np.int32)
        ca = np.ascontiguousarray(ca, np.int32)
        cb = np.ascontiguousarray(cb, np.int32)
        out = np.zeros_like(ca)
        self.lib.orc_boots_gate_exact_batch(ctypes.byref(P), _p(np.ascontiguousarray(bk, np.int32), I32P),
                                            _p(ks, I32P), _p(gates, I32P), _p(ca, I32P), _p(cb, I32P),
                                            _p(out, I32P), len(gates), int(threads))
        return out


class CpuFast:
    """The faster CPU gate bootstrap (oracle/tfhe_cpu_fast.cpp): the same
    gates with the N/2-point twisted transform in double precision, for the
    timed CPU comparison only.  Holds the key in its transform domain; the
    key-switching key array is referenced, not copied, and is kept alive
    here."""

    def __init__(self, P, bk, ks, lib_path=None):
        if lib_path is None:
            lib_path = build_oracle.build_fast()
        self.lib = ctypes.CDLL(lib_path)
        self.lib.cpuf_create.restype = ctypes.c_void_p
        self.lib.cpuf_create.argtypes = [ctypes.POINTER(Params), I32P, I32P]
        self.lib.cpuf_destroy.restype = None
        self.lib.cpuf_destroy.argtypes = [ctypes.c_void_p]
        self.lib.cpuf_boots_gates.restype = None
        self.lib.cpuf_boots_gates.argtypes = [ctypes.c_void_p, I32P, I32P, I32P, I32P, ctypes.c_int32,
                                              ctypes.c_int32]
        self.P = P
        self._ks = np.ascontiguousarray(ks, np.int32)
        bk = np.ascontiguousarray(bk, np.int32)
        self.h = self.lib.cpuf_create(ctypes.byref(P), _p(bk, I32P), _p(self._ks, I32P))
        if not self.h:
            raise ValueError("cpuf_create refused the parameters")

    def boots_gates(self, gates, ca, cb, threads=0):
        gates = np.ascontiguousarray(gates, np.int32)
        ca = np.ascontiguousarray(ca, np.int32)
        cb = np.ascontiguousarray(cb, np.int32)
        out = np.zeros_like(ca)
        self.lib.cpuf_boots_gates(self.h, _p(gates, I32P), _p(ca, I32P), _p(cb, I32P), _p(out, I32P),
                                  len(gates), int(threads))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpuf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ORACLE = None


def get():
    global _ORACLE
    if _ORACLE is None:
        _ORACLE = Oracle()
    return _ORACLE
