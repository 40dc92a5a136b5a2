/*
 * tfhe_oracle.h -- CPU oracle for the TFHE gate-bootstrapping path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference leg of bench.py may load this library.  The
 * product (the CUDA engine and its host code) never links or calls it.
 *
 * It restates, on the CPU, the algorithm of the reference's FPGA port
 * (shreks99/fpga-tfhe) and of the upstream TFHE library that the port calls
 * but does not vendor (the `tfhe/` submodule is empty; no version is pinned).
 * Every function cites the reference file:line it follows; functions that
 * exist only upstream restate the published TFHE algorithm (Chillotti, Gama,
 * Georgieva, Izabachene, J. Cryptology 2020) and say so.
 *
 * Parity pins: tests/test_oracle_vs_reference.py compares this restatement
 * function by function with the reference's own sources compiled on the CPU
 * (oracle/ref_pin/build_ref.py -> oracle/_ref/): bit-exact for the integer
 * functions, RNG and key switch, within 1-2 units for the FFT path.
 * tests/test_oracle_pins.py holds the known answers (mu = 2^29, the offset
 * 2164391936, 499 OR 388 = 503 from test_bench/).  The upstream-only pieces
 * (TLWE/TGSW keygen, extraction, gate constants other than OR) are not
 * pinned: the upstream library is absent.
 *
 * Layouts (all int32 arrays are Torus32 values, arithmetic mod 2^32):
 *   LWE sample         : int32[n + 1]            a[0..n-1], b
 *   TLWE sample        : int32[(k+1) * N]        a[0..k-1], b = a[k]
 *   TGSW sample        : int32[kpl * (k+1) * N]  row p = i*l + j
 *   Lagrange half poly : double[N/2][2]          values at w^(2m+1), w = e^{i pi/N}
 *   TGSW in FFT domain : double[kpl][(k+1)][N/2][2]
 *   bootstrapping key  : n TGSW samples
 *   key-switching key  : int32[kN][t][base][n + 1]
 */
#ifndef TFHE_ORACLE_H
#define TFHE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t n;          /* LWE dimension                              */
    int32_t N;          /* ring degree                                */
    int32_t k;          /* TLWE mask polynomials                      */
    int32_t l;          /* gadget decomposition length                */
    int32_t Bgbit;      /* log2 of the decomposition base             */
    int32_t ks_t;       /* key-switch decomposition length            */
    int32_t ks_basebit; /* log2 of the key-switch base                */
    int32_t pad_;
    double lwe_alpha;   /* LWE noise stdev (also the KS key noise)    */
    double tlwe_alpha;  /* TLWE/TGSW noise stdev (bootstrapping key)  */
} orc_params;

/* ---- random generator (numeric-functions.cpp:11-34) ---------------- */
void orc_set_seed(const uint32_t* values, int32_t size);
int32_t orc_uniform_torus32(void);
int32_t orc_gaussian32(int32_t message, double sigma);
int32_t orc_dtot32(double d);

/* ---- numeric functions (numeric-functions.cpp:45-76) --------------- */
int32_t orc_mod_switch_from_torus32(int32_t phase, int32_t Msize);
int32_t orc_mod_switch_to_torus32(int32_t mu, int32_t Msize);
int32_t orc_approx_phase(int32_t phase, int32_t Msize);

/* ---- LWE (lwe-functions.cpp) ---------------------------------------- */
void orc_lwe_keygen(int32_t* key, int32_t n);
void orc_lwe_encrypt(int32_t* out, int32_t message, double alpha,
                     const int32_t* key, int32_t n);
int32_t orc_lwe_phase(const int32_t* sample, const int32_t* key, int32_t n);

/* ---- key generation (upstream; restated) ---------------------------- */
void orc_tlwe_keygen(int32_t* key, int32_t k, int32_t N);
void orc_tgsw_encrypt_int(const orc_params* P, int32_t* out, int32_t message,
                          double alpha, const int32_t* tlwe_key);
void orc_create_ks_key(const orc_params* P, int32_t* ks, const int32_t* in_key,
                       int32_t n_in, const int32_t* out_key);
/* new_random_gate_bootstrapping_secret_keyset: LWE key, TLWE key, KS, BK */
void orc_gate_keyset(const orc_params* P, int32_t* lwe_key, int32_t* tlwe_key,
                     int32_t* ks, int32_t* bk);

/* bootsSymEncrypt / bootsSymDecrypt (upstream; restated) */
void orc_boots_sym_encrypt(const orc_params* P, int32_t* out, int32_t bit,
                           const int32_t* lwe_key);
int32_t orc_boots_sym_decrypt(const orc_params* P, const int32_t* sample,
                              const int32_t* lwe_key);

/* ---- hot path pieces ------------------------------------------------ */
void orc_decompose(const orc_params* P, const int32_t* poly, int32_t* out);
void orc_int_poly_ifft(int32_t N, const int32_t* poly, double* out);
void orc_torus_poly_ifft(int32_t N, const int32_t* poly, double* out);
void orc_torus_poly_fft(int32_t N, const double* in, int32_t* out);
void orc_tgsw_to_fft(const orc_params* P, const int32_t* tgsw, double* out);
void orc_bk_to_fft(const orc_params* P, const int32_t* bk, double* out);

void orc_mul_by_xai(int32_t N, int32_t a, const int32_t* in, int32_t* out);
void orc_mul_by_xai_minus_one(int32_t N, int32_t a, const int32_t* in,
                              int32_t* out);
void orc_extern_mul_fft(const orc_params* P, int32_t* accum,
                        const double* gsw_fft);
void orc_extern_mul_exact(const orc_params* P, int32_t* accum,
                          const int32_t* gsw);
void orc_mux_rotate_fft(const orc_params* P, int32_t* result,
                        const int32_t* accum, const double* bki_fft,
                        int32_t barai);
void orc_blind_rotate_fft(const orc_params* P, int32_t* accum,
                          const double* bk_fft, const int32_t* bara);
void orc_blind_rotate_exact(const orc_params* P, int32_t* accum,
                            const int32_t* bk, const int32_t* bara);
void orc_extract(const orc_params* P, const int32_t* accum, int32_t* out);
void orc_keyswitch(const orc_params* P, const int32_t* ks, const int32_t* in,
                   int32_t* out);

/* bootstrap front end: bara/barb and the rotated test vector */
void orc_bootstrap_prologue(const orc_params* P, int32_t mu, const int32_t* x,
                            int32_t* bara, int32_t* accum);
/* tfhe_bootstrap_woKS_FFT: x (LWE n) -> extracted LWE (kN) */
void orc_bootstrap_woks(const orc_params* P, const double* bk_fft, int32_t mu,
                        const int32_t* x, int32_t* out, int32_t exact,
                        const int32_t* bk);

/* Programmable bootstrap: test vector tv (N int32) instead of the constant
 * mu; with key switch.  _batch: count items, tv_stride int32 apart (0 = one
 * shared vector), on `threads` OpenMP threads. */
void orc_bootstrap_tv(const orc_params* P, const double* bk_fft, const int32_t* ks,
                      const int32_t* tv, const int32_t* x, int32_t* out);
void orc_bootstrap_tv_batch(const orc_params* P, const double* bk_fft, const int32_t* ks,
                            const int32_t* tv, int32_t tv_stride, const int32_t* x,
                            int32_t* out, int32_t count, int32_t threads);
/* test vector of a lookup table on p padded messages (m at phase m/(2p)) */
void orc_test_vector(int32_t N, const int32_t* table, int32_t p, int32_t* tv);

/* Gate identifiers (shared with the engine's public header). */
enum {
    ORC_GATE_NAND = 0, ORC_GATE_AND = 1, ORC_GATE_OR = 2, ORC_GATE_XOR = 3,
    ORC_GATE_XNOR = 4, ORC_GATE_NOR = 5, ORC_GATE_ANDNY = 6,
    ORC_GATE_ANDYN = 7, ORC_GATE_ORNY = 8, ORC_GATE_ORYN = 9
};
/* gate linear combination (tfhe_blindRotate_FFT_tb.cpp:267-276 for OR) */
void orc_gate_combine(const orc_params* P, int32_t gate, const int32_t* ca,
                      const int32_t* cb, int32_t* out);
/* full gate: combine, bootstrap, key switch */
void orc_boots_gate(const orc_params* P, const double* bk_fft,
                    const int32_t* ks, int32_t gate, const int32_t* ca,
                    const int32_t* cb, int32_t* out);
/* bootsMUX (cloud.c:11): two bootstraps without KS, add, one KS */
void orc_boots_mux(const orc_params* P, const double* bk_fft,
                   const int32_t* ks, const int32_t* a, const int32_t* b,
                   const int32_t* c, int32_t* out);
/* count independent bootsMUX on `threads` OpenMP threads (<= 0: all). */
void orc_boots_mux_batch(const orc_params* P, const double* bk_fft,
                         const int32_t* ks, const int32_t* a, const int32_t* b,
                         const int32_t* c, int32_t* out, int32_t count,
                         int32_t threads);
/* a batch of independent gates on `threads` OpenMP threads */
void orc_boots_gate_batch(const orc_params* P, const double* bk_fft,
                          const int32_t* ks, const int32_t* gates,
                          const int32_t* ca, const int32_t* cb, int32_t* out,
                          int32_t count, int32_t threads);
/* independent exact external products (time-domain TGSW per item) */
void orc_extern_mul_exact_batch(const orc_params* P, int32_t* accum, const int32_t* gsw,
                                int32_t count, int32_t threads);
/* bootstraps without key switch of a batch; exact != 0: int64 blind
 * rotation with the time-domain key bk */
void orc_bootstrap_woks_batch(const orc_params* P, const double* bk_fft, int32_t mu,
                              const int32_t* x, int32_t* out, int32_t count,
                              int32_t exact, const int32_t* bk, int32_t threads);
/* a batch of gates through the exact int64 blind rotation */
void orc_boots_gate_exact_batch(const orc_params* P, const int32_t* bk,
                                const int32_t* ks, const int32_t* gates,
                                const int32_t* ca, const int32_t* cb, int32_t* out,
                                int32_t count, int32_t threads);
int32_t orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
