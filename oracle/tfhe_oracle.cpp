/*
 * tfhe_oracle.cpp -- CPU oracle for the TFHE gate-bootstrapping path.
 *
 * TEST INFRASTRUCTURE ONLY (see tfhe_oracle.h).  Nothing in the engine
 * links this file; tests and the CPU-baseline leg of bench.py load it.
 *
 * Reference citations are paths inside shreks99/fpga-tfhe.  "Upstream"
 * means the TFHE library the reference links (-ltfhe-spqlios-fma /
 * -ltfhe-nayuki-portable, test_bench/Makefile:6) whose sources are not in
 * the reference (the tfhe/ submodule is empty, no version pinned); those
 * pieces restate the published TFHE algorithm in this file's own code.
 *
 * Integer semantics: Torus32 arithmetic wraps mod 2^32.  It is done on
 * uint32_t here so that the wrap is defined behaviour in C++.
 */
#include "tfhe_oracle.h"

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits.h>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cplx;

/* numeric-functions.cpp:11-12: one global engine, one global uniform
 * distribution over the full int32 range. */
std::default_random_engine g_gen;
std::uniform_int_distribution<int32_t> g_unif_torus(INT32_MIN, INT32_MAX);

inline int32_t wrap_add(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a + (uint32_t)b);
}
inline int32_t wrap_sub(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a - (uint32_t)b);
}
inline int32_t wrap_mul(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}

/* ------------------------------------------------------------------ */
/* 2N-point complex DFT, forward sign e^{-2 pi i jk / M}.  The reference */
/* uses the SPIRAL Pease FFT for this (tfhe_blindRotate_FFT/            */
/* pease_fft.cpp:660-717, twiddles include/twidR.txt, twidI.txt: the    */
/* table holds cos(2 pi k/2048), -sin(2 pi k/2048)).  This is an        */
/* independent iterative radix-2 transform computing the same DFT.      */
/* ------------------------------------------------------------------ */
struct Fft {
    int M = 0;
    int logM = 0;
    std::vector<int> rev;
    std::vector<double> wr, wi; /* e^{-2 pi i k / M}, k < M/2 */

    void init(int m) {
        M = m;
        logM = 0;
        while ((1 << logM) < M) ++logM;
        rev.assign(M, 0);
        for (int i = 0; i < M; ++i) {
            int r = 0;
            for (int b = 0; b < logM; ++b)
                if (i & (1 << b)) r |= 1 << (logM - 1 - b);
            rev[i] = r;
        }
        wr.resize(M / 2);
        wi.resize(M / 2);
        for (int k = 0; k < M / 2; ++k) {
            /* exact symmetric reduction: angle = 2 pi k / M */
            double c, s;
            sincos_2pi_frac(k, M, &c, &s);
            wr[k] = c;
            wi[k] = -s;
        }
    }

    /* cos/sin of 2 pi k/M using octant symmetry so that the table is
     * exactly symmetric (the reference's table is symmetric too). */
    static void sincos_2pi_frac(int k, int M, double* c, double* s) {
        k %= M;
        int q = (4 * k) / M;            /* quadrant */
        int r = k - q * (M / 4);        /* 0 <= r < M/4 */
        double cr, sr;
        if (8 * r <= M) {
            double a = 2.0 * M_PI * (double)r / (double)M;
            cr = std::cos(a);
            sr = std::sin(a);
        } else {
            double a = 2.0 * M_PI * (double)(M / 4 - r) / (double)M;
            cr = std::sin(a);
            sr = std::cos(a);
        }
        switch (q) {
        case 0: *c = cr; *s = sr; break;
        case 1: *c = -sr; *s = cr; break;
        case 2: *c = -cr; *s = -sr; break;
        default: *c = sr; *s = -cr; break;
        }
    }

    /* in place, natural order in and out */
    void forward(double* re, double* im) const {
        for (int i = 0; i < M; ++i) {
            int r = rev[i];
            if (r > i) {
                std::swap(re[i], re[r]);
                std::swap(im[i], im[r]);
            }
        }
        for (int half = 1; half < M; half <<= 1) {
            const int step = M / (2 * half);
            for (int base = 0; base < M; base += 2 * half) {
                for (int j = 0; j < half; ++j) {
                    const double c = wr[j * step], s = wi[j * step];
                    const int u = base + j, v = u + half;
                    const double tr = re[v] * c - im[v] * s;
                    const double ti = re[v] * s + im[v] * c;
                    re[v] = re[u] - tr;
                    im[v] = im[u] - ti;
                    re[u] = re[u] + tr;
                    im[u] = im[u] + ti;
                }
            }
        }
    }
};

Fft& fft_for(int M) {
    /* one table per size; sizes used here are 2N (2048) only */
    static thread_local Fft f;
    if (f.M != M) f.init(M);
    return f;
}

/* IntPolynomial -> LagrangeHalfC, following the correct `ifft` of
 * tGswFFTExternMulToTLwe.cpp:97-130: antiperiodic extension with c/2,
 * forward 2N-point DFT, conjugate, keep odd bins 1, 3, ..., N-1.  The
 * result is P(w^(2m+1)), w = e^{i pi / N}, m < N/2.  `scale` is 1/2 for
 * integer polynomials and 2^-33 for Torus32 (upstream execute_reverse_
 * torus32, restated: torus value / 2^32, halved by the same extension). */
void to_lagrange(int N, const int32_t* poly, double scale, double* out) {
    const int M = 2 * N;
    std::vector<double> re(M), im(M, 0.0);
    for (int i = 0; i < N; ++i) {
        re[i] = (double)poly[i] * scale;
        re[N + i] = -re[i];
    }
    fft_for(M).forward(re.data(), im.data());
    for (int m = 0; m < N / 2; ++m) {
        out[2 * m] = re[2 * m + 1];
        out[2 * m + 1] = -im[2 * m + 1];
    }
}

}  // namespace

extern "C" {

/* ---------------- random generator: numeric-functions.cpp ---------- */

/* numeric-functions.cpp:16-19 */
void orc_set_seed(const uint32_t* values, int32_t size) {
    std::seed_seq seeds(values, values + size);
    g_gen.seed(seeds);
}

int32_t orc_uniform_torus32(void) { return g_unif_torus(g_gen); }

/* numeric-functions.cpp:32-34 */
int32_t orc_dtot32(double d) {
    return (int32_t)(int64_t)((d - (double)(int64_t)d) * 4294967296.0);
}

/* numeric-functions.cpp:22-27: a fresh normal_distribution per call (the
 * cached second variate of the polar method is dropped on purpose). */
int32_t orc_gaussian32(int32_t message, double sigma) {
    std::normal_distribution<double> distribution(0., sigma);
    double err = distribution(g_gen);
    return wrap_add(message, orc_dtot32(err));
}

/* numeric-functions.cpp:59-65 (dup. include/host_constants.h:39-45,
 * tfhe_bootstrap_woKS_FFT.cpp:3-10) */
int32_t orc_mod_switch_from_torus32(int32_t phase, int32_t Msize) {
    uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    uint64_t half_interval = interv / 2;
    uint64_t phase64 = ((uint64_t)(int64_t)phase << 32) + half_interval;
    return (int32_t)(phase64 / interv);
}

/* numeric-functions.cpp:71-76 */
int32_t orc_mod_switch_to_torus32(int32_t mu, int32_t Msize) {
    uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    uint64_t phase64 = (uint64_t)(int64_t)mu * interv;
    return (int32_t)(phase64 >> 32);
}

/* numeric-functions.cpp:45-53 */
int32_t orc_approx_phase(int32_t phase, int32_t Msize) {
    uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    uint64_t half_interval = interv / 2;
    uint64_t phase64 = ((uint64_t)(int64_t)phase << 32) + half_interval;
    phase64 -= phase64 % interv;
    return (int32_t)(phase64 >> 32);
}

/* ---------------- LWE: lwe-functions.cpp ---------------------------- */

/* lwe-functions.cpp:21-27 */
void orc_lwe_keygen(int32_t* key, int32_t n) {
    std::uniform_int_distribution<int32_t> distribution(0, 1);
    for (int32_t i = 0; i < n; i++) key[i] = distribution(g_gen);
}

/* lwe-functions.cpp:36-47 */
void orc_lwe_encrypt(int32_t* out, int32_t message, double alpha,
                     const int32_t* key, int32_t n) {
    int32_t b = orc_gaussian32(message, alpha);
    for (int32_t i = 0; i < n; ++i) {
        out[i] = g_unif_torus(g_gen);
        b = wrap_add(b, wrap_mul(out[i], key[i]));
    }
    out[n] = b;
}

/* lwe-functions.cpp:53-64 */
static void lwe_encrypt_external_noise(int32_t* out, int32_t message,
                                       double noise, const int32_t* key,
                                       int32_t n) {
    int32_t b = wrap_add(message, orc_dtot32(noise));
    for (int32_t i = 0; i < n; ++i) {
        out[i] = g_unif_torus(g_gen);
        b = wrap_add(b, wrap_mul(out[i], key[i]));
    }
    out[n] = b;
}

/* lwe-functions.cpp:72-81 */
int32_t orc_lwe_phase(const int32_t* sample, const int32_t* key, int32_t n) {
    uint32_t axs = 0;
    for (int32_t i = 0; i < n; ++i)
        axs += (uint32_t)sample[i] * (uint32_t)key[i];
    return (int32_t)((uint32_t)sample[n] - axs);
}

/* ---------------- key generation (upstream, restated) --------------- */

/* upstream tLweKeyGen: k*N draws of uniform_int_distribution(0,1) */
void orc_tlwe_keygen(int32_t* key, int32_t k, int32_t N) {
    std::uniform_int_distribution<int32_t> distribution(0, 1);
    for (int32_t i = 0; i < k; ++i)
        for (int32_t j = 0; j < N; ++j) key[i * N + j] = distribution(g_gen);
}

/* exact negacyclic  res += key * a  (key binary/int, a Torus32) */
static void poly_addmul_exact(int32_t N, int32_t* res, const int32_t* key,
                              const int32_t* a) {
    std::vector<uint32_t> acc(N, 0);
    for (int32_t j = 0; j < N; ++j) {
        const uint32_t kj = (uint32_t)key[j];
        if (kj == 0) continue;
        for (int32_t i = 0; i < j; ++i) acc[i] -= kj * (uint32_t)a[i - j + N];
        for (int32_t i = j; i < N; ++i) acc[i] += kj * (uint32_t)a[i - j];
    }
    for (int32_t i = 0; i < N; ++i) res[i] = (int32_t)((uint32_t)res[i] + acc[i]);
}

/* upstream tLweSymEncryptZero: b_j = gaussian32(0, alpha) for j < N, then
 * for each mask polynomial: N uniform Torus32 draws and b += key_i * a_i.
 * The key product is exact (upstream may use an FFT product whose int64
 * truncation can move a coefficient by one unit; that is not reproduced). */
static void tlwe_encrypt_zero(int32_t N, int32_t k, int32_t* sample,
                              double alpha, const int32_t* tlwe_key) {
    int32_t* b = sample + k * N;
    for (int32_t j = 0; j < N; ++j) b[j] = orc_gaussian32(0, alpha);
    for (int32_t i = 0; i < k; ++i) {
        int32_t* a = sample + i * N;
        for (int32_t j = 0; j < N; ++j) a[j] = g_unif_torus(g_gen);
        poly_addmul_exact(N, b, tlwe_key + i * N, a);
    }
}

/* upstream tGswSymEncryptInt = tGswEncryptZero + tGswAddMuIntH:
 * row (i, j) gets message * h_j added to coefficient 0 of polynomial i,
 * h_j = 2^(32 - (j+1) Bgbit). */
void orc_tgsw_encrypt_int(const orc_params* P, int32_t* out, int32_t message,
                          double alpha, const int32_t* tlwe_key) {
    const int32_t N = P->N, k = P->k, l = P->l;
    const int32_t kpl = (k + 1) * l;
    for (int32_t p = 0; p < kpl; ++p)
        tlwe_encrypt_zero(N, k, out + (size_t)p * (k + 1) * N, alpha, tlwe_key);
    for (int32_t i = 0; i <= k; ++i)
        for (int32_t j = 0; j < l; ++j) {
            const uint32_t h = 1u << (32 - (j + 1) * P->Bgbit);
            int32_t* row = out + (size_t)(i * l + j) * (k + 1) * N;
            row[i * N] = (int32_t)((uint32_t)row[i * N] + (uint32_t)message * h);
        }
}

/* lwe-keyswitch-functions.cpp:163-215 (lweCreateKeySwitchKey): draw all
 * n_in*t*(base-1) Gaussian noises first, recentre them, then encrypt
 * h * s_i / base^(j+1) with that external noise; h = 0 is a trivial 0. */
void orc_create_ks_key(const orc_params* P, int32_t* ks, const int32_t* in_key,
                       int32_t n_in, const int32_t* out_key) {
    const int32_t t = P->ks_t, basebit = P->ks_basebit, base = 1 << basebit;
    const int32_t n = P->n;
    const double alpha = P->lwe_alpha;
    const int32_t sizeks = n_in * t * (base - 1);
    std::vector<double> noise(sizeks);
    double err = 0;
    for (int32_t i = 0; i < sizeks; ++i) {
        std::normal_distribution<double> distribution(0., alpha);
        noise[i] = distribution(g_gen);
        err += noise[i];
    }
    err = err / sizeks;
    for (int32_t i = 0; i < sizeks; ++i) noise[i] -= err;
    int32_t index = 0;
    for (int32_t i = 0; i < n_in; ++i)
        for (int32_t j = 0; j < t; ++j) {
            int32_t* row0 = ks + ((size_t)(i * t + j) * base) * (n + 1);
            std::memset(row0, 0, sizeof(int32_t) * (n + 1));
            for (int32_t h = 1; h < base; ++h) {
                const uint32_t mess = (uint32_t)in_key[i] * (uint32_t)h *
                                      (1u << (32 - (j + 1) * basebit));
                lwe_encrypt_external_noise(row0 + (size_t)h * (n + 1),
                                           (int32_t)mess, noise[index],
                                           out_key, n);
                index += 1;
            }
        }
}

/* upstream new_random_gate_bootstrapping_secret_keyset:
 * lweKeyGen, tGswKeyGen, then tfhe_createLweBootstrappingKey: the KS key
 * from the extracted TLWE key to the LWE key, then BK_i = TGSW(s_i). */
void orc_gate_keyset(const orc_params* P, int32_t* lwe_key, int32_t* tlwe_key,
                     int32_t* ks, int32_t* bk) {
    const int32_t n = P->n, N = P->N, k = P->k, l = P->l;
    const size_t tgsw_words = (size_t)(k + 1) * l * (k + 1) * N;
    orc_lwe_keygen(lwe_key, n);
    orc_tlwe_keygen(tlwe_key, k, N);
    /* tLweExtractKey: extracted[i*N + j] = key_i[j] */
    orc_create_ks_key(P, ks, tlwe_key, k * N, lwe_key);
    for (int32_t i = 0; i < n; ++i)
        orc_tgsw_encrypt_int(P, bk + i * tgsw_words, lwe_key[i], P->tlwe_alpha,
                             tlwe_key);
}

/* upstream bootsSymEncrypt: mu = +-1/8, alpha = LWE alpha_min */
void orc_boots_sym_encrypt(const orc_params* P, int32_t* out, int32_t bit,
                           const int32_t* lwe_key) {
    const int32_t s8 = orc_mod_switch_to_torus32(1, 8);
    const int32_t mu = bit ? s8 : -s8;
    orc_lwe_encrypt(out, mu, P->lwe_alpha, lwe_key, P->n);
}

/* upstream bootsSymDecrypt: phase > 0 */
int32_t orc_boots_sym_decrypt(const orc_params* P, const int32_t* sample,
                              const int32_t* lwe_key) {
    return orc_lwe_phase(sample, lwe_key, P->n) > 0 ? 1 : 0;
}

/* ---------------- hot path ------------------------------------------ */

/* tGswFFTExternMulToTLwe.cpp:76-95 (decompose) and
 * tGswTorus32PolynomialDecompH.cpp:29-44: add the offset
 * sum_p halfBg 2^(32-(p+1)Bgbit) (2164391936 for l=3, Bgbit=7,
 * constants.h:24), take Bgbit-bit digits, subtract halfBg. */
void orc_decompose(const orc_params* P, const int32_t* poly, int32_t* out) {
    const int32_t N = P->N, l = P->l, Bgbit = P->Bgbit;
    const int32_t halfBg = 1 << (Bgbit - 1);
    const uint32_t maskMod = (1u << Bgbit) - 1;
    uint32_t offset = 0;
    for (int32_t i = 0; i < l; ++i) offset += 1u << (32 - (i + 1) * Bgbit);
    offset *= (uint32_t)halfBg;
    for (int32_t p = 0; p < l; ++p) {
        const int32_t decal = 32 - (p + 1) * Bgbit;
        for (int32_t j = 0; j < N; ++j) {
            const uint32_t u = (uint32_t)poly[j] + offset;
            out[p * N + j] = (int32_t)((u >> decal) & maskMod) - halfBg;
        }
    }
}

void orc_int_poly_ifft(int32_t N, const int32_t* poly, double* out) {
    to_lagrange(N, poly, 0.5, out);
}

void orc_torus_poly_ifft(int32_t N, const int32_t* poly, double* out) {
    to_lagrange(N, poly, 1.0 / 8589934592.0, out);
}

/* TorusPolynomial_fft.cpp:4-43: Hermitian placement on the odd bins,
 * forward 2N-point DFT, Torus32(int64(re * (1/N) * 2^32)) -- truncating. */
void orc_torus_poly_fft(int32_t N, const double* in, int32_t* out) {
    const int M = 2 * N;
    const double two32 = 4294967296.0;
    const double inv_n = 1.0 / (double)N;
    std::vector<double> re(M, 0.0), im(M, 0.0);
    for (int i = 0; i < N / 2; ++i) {
        re[2 * i + 1] = in[2 * i];
        im[2 * i + 1] = in[2 * i + 1];
        re[M - 1 - 2 * i] = in[2 * i];
        im[M - 1 - 2 * i] = -in[2 * i + 1];
    }
    fft_for(M).forward(re.data(), im.data());
    for (int i = 0; i < N; ++i)
        out[i] = (int32_t)(uint32_t)(uint64_t)(int64_t)(re[i] * inv_n * two32);
}

/* upstream tGswToFftConvert: every polynomial of every row */
void orc_tgsw_to_fft(const orc_params* P, const int32_t* tgsw, double* out) {
    const int32_t N = P->N, k = P->k, kpl = (k + 1) * P->l;
    for (int32_t p = 0; p < kpl; ++p)
        for (int32_t j = 0; j <= k; ++j)
            orc_torus_poly_ifft(N, tgsw + (size_t)(p * (k + 1) + j) * N,
                                out + (size_t)(p * (k + 1) + j) * N);
}

void orc_bk_to_fft(const orc_params* P, const int32_t* bk, double* out) {
    const size_t words = (size_t)(P->k + 1) * P->l * (P->k + 1) * P->N;
    for (int32_t i = 0; i < P->n; ++i)
        orc_tgsw_to_fft(P, bk + i * words, out + i * words);
}

/* upstream torusPolynomialMulByXai; same as mulByXaiOrCopy.cpp:25-41 */
void orc_mul_by_xai(int32_t N, int32_t a, const int32_t* in, int32_t* out) {
    if (a < N) {
        for (int32_t i = 0; i < a; i++) out[i] = wrap_sub(0, in[i - a + N]);
        for (int32_t i = a; i < N; i++) out[i] = in[i - a];
    } else {
        const int32_t aa = a - N;
        for (int32_t i = 0; i < aa; i++) out[i] = in[i - aa + N];
        for (int32_t i = aa; i < N; i++) out[i] = wrap_sub(0, in[i - aa]);
    }
}

/* tfhe_MuxRotate_FFT.cpp:5-24 */
void orc_mul_by_xai_minus_one(int32_t N, int32_t a, const int32_t* in,
                              int32_t* out) {
    if (a < N) {
        for (int32_t i = 0; i < a; i++)
            out[i] = wrap_sub(wrap_sub(0, in[i - a + N]), in[i]);
        for (int32_t i = a; i < N; i++) out[i] = wrap_sub(in[i - a], in[i]);
    } else {
        const int32_t aa = a - N;
        for (int32_t i = 0; i < aa; i++) out[i] = wrap_sub(in[i - aa + N], in[i]);
        for (int32_t i = aa; i < N; i++)
            out[i] = wrap_sub(wrap_sub(0, in[i - aa]), in[i]);
    }
}

/* tGswFFTExternMulToTLwe.cpp:203-247 (the correct _FPGA form): decompose
 * each of the k+1 polynomials, transform the kpl digit polynomials, clear,
 * multiply-accumulate against the TGSW rows (:166-197), transform back
 * (tLweFromFFTConvert.cpp:4-24).  accum is overwritten. */
void orc_extern_mul_fft(const orc_params* P, int32_t* accum,
                        const double* gsw_fft) {
    const int32_t N = P->N, k = P->k, l = P->l, kpl = (k + 1) * l;
    const int32_t Ns2 = N / 2;
    std::vector<int32_t> deca((size_t)kpl * N);
    std::vector<double> decaFFT((size_t)kpl * N);
    for (int32_t i = 0; i <= k; ++i)
        orc_decompose(P, accum + i * N, deca.data() + (size_t)i * l * N);
    for (int32_t p = 0; p < kpl; ++p)
        orc_int_poly_ifft(N, deca.data() + (size_t)p * N,
                          decaFFT.data() + (size_t)p * N);
    std::vector<double> tmpa((size_t)(k + 1) * N, 0.0);
    for (int32_t p = 0; p < kpl; ++p) {
        const double* d = decaFFT.data() + (size_t)p * N;
        for (int32_t j = 0; j <= k; ++j) {
            const double* g = gsw_fft + (size_t)(p * (k + 1) + j) * N;
            double* t = tmpa.data() + (size_t)j * N;
            for (int32_t m = 0; m < Ns2; ++m) {
                const double ar = d[2 * m], ai = d[2 * m + 1];
                const double br = g[2 * m], bi = g[2 * m + 1];
                t[2 * m] += ar * br - ai * bi;
                t[2 * m + 1] += ar * bi + ai * br;
            }
        }
    }
    for (int32_t j = 0; j <= k; ++j)
        orc_torus_poly_fft(N, tmpa.data() + (size_t)j * N, accum + j * N);
}

/* The same product computed exactly: sum_p D_p * K_{p,j} negacyclic over
 * the integers, reduced mod 2^32.  This is the "int64 negacyclic-product
 * oracle".  The sums are carried in wrapping uint32 arithmetic: reduction
 * mod 2^32 commutes with every + and x, so each word equals the int64 sum
 * reduced at the end, bit for bit, and the loops vectorise on 32-bit lanes. */
void orc_extern_mul_exact(const orc_params* P, int32_t* accum,
                          const int32_t* gsw) {
    const int32_t N = P->N, k = P->k, l = P->l, kpl = (k + 1) * l;
    std::vector<int32_t> deca((size_t)kpl * N);
    for (int32_t i = 0; i <= k; ++i)
        orc_decompose(P, accum + i * N, deca.data() + (size_t)i * l * N);
    std::vector<uint32_t> acc((size_t)(k + 1) * N, 0);
    std::vector<int32_t> nz;
    for (int32_t p = 0; p < kpl; ++p) {
        const int32_t* d = deca.data() + (size_t)p * N;
        for (int32_t j = 0; j <= k; ++j) {
            const uint32_t* g = reinterpret_cast<const uint32_t*>(gsw) + (size_t)(p * (k + 1) + j) * N;
            uint32_t* o = acc.data() + (size_t)j * N;
            nz.clear();
            for (int32_t t = 0; t < N && (int32_t)nz.size() * 8 <= N; ++t)
                if (g[t]) nz.push_back(t);
            if ((int32_t)nz.size() * 8 <= N) {
                /* sparse key polynomial (e.g. a noiseless trivial TGSW):
                 * the same sum, taken over its non-zero terms */
                for (int32_t t : nz) {
                    const uint32_t gt = g[t];
                    for (int32_t i = 0; i < N - t; ++i) o[i + t] += (uint32_t)d[i] * gt;
                    for (int32_t i = N - t; i < N; ++i) o[i + t - N] -= (uint32_t)d[i] * gt;
                }
                continue;
            }
            for (int32_t s = 0; s < N; ++s) {
                const uint32_t ds = (uint32_t)d[s];
                if (ds == 0) continue;
                for (int32_t i = 0; i < s; ++i) o[i] -= ds * g[i - s + N];
                for (int32_t i = s; i < N; ++i) o[i] += ds * g[i - s];
            }
        }
    }
    for (int32_t i = 0; i < (k + 1) * N; ++i)
        accum[i] = (int32_t)acc[i];
}

/* tfhe_MuxRotate_FFT.cpp:56-85: result = BK_i [(X^a - 1) acc] + acc.
 * tLweAddTo_FPGA (:48-54) also copies a[k] into the duplicate b; here the
 * TLWE layout has no duplicate, b is a[k]. */
void orc_mux_rotate_fft(const orc_params* P, int32_t* result,
                        const int32_t* accum, const double* bki_fft,
                        int32_t barai) {
    const int32_t N = P->N, k = P->k;
    for (int32_t i = 0; i <= k; ++i)
        orc_mul_by_xai_minus_one(N, barai, accum + i * N, result + i * N);
    orc_extern_mul_fft(P, result, bki_fft);
    for (int32_t i = 0; i < (k + 1) * N; ++i)
        result[i] = wrap_add(result[i], accum[i]);
}

static void mux_rotate_exact(const orc_params* P, int32_t* result,
                             const int32_t* accum, const int32_t* bki,
                             int32_t barai) {
    const int32_t N = P->N, k = P->k;
    for (int32_t i = 0; i <= k; ++i)
        orc_mul_by_xai_minus_one(N, barai, accum + i * N, result + i * N);
    orc_extern_mul_exact(P, result, bki);
    for (int32_t i = 0; i < (k + 1) * N; ++i)
        result[i] = wrap_add(result[i], accum[i]);
}

/* tfhe_blindRotate_FFT.cpp:61-147 with the loop over all n steps (the
 * reference's loop bound at :112 runs one step only; the CPU reference it
 * compares against, tb:325, runs all n) and the skip of bara_i == 0 (:114). */
void orc_blind_rotate_fft(const orc_params* P, int32_t* accum,
                          const double* bk_fft, const int32_t* bara) {
    const int32_t N = P->N, k = P->k, kpl = (k + 1) * P->l;
    const size_t words = (size_t)kpl * (k + 1) * N;
    std::vector<int32_t> tmp((size_t)(k + 1) * N);
    for (int32_t i = 0; i < P->n; ++i) {
        if (bara[i] == 0) continue;
        orc_mux_rotate_fft(P, tmp.data(), accum, bk_fft + i * words, bara[i]);
        std::memcpy(accum, tmp.data(), sizeof(int32_t) * tmp.size());
    }
}

void orc_blind_rotate_exact(const orc_params* P, int32_t* accum,
                            const int32_t* bk, const int32_t* bara) {
    const int32_t N = P->N, k = P->k, kpl = (k + 1) * P->l;
    const size_t words = (size_t)kpl * (k + 1) * N;
    std::vector<int32_t> tmp((size_t)(k + 1) * N);
    for (int32_t i = 0; i < P->n; ++i) {
        if (bara[i] == 0) continue;
        mux_rotate_exact(P, tmp.data(), accum, bk + i * words, bara[i]);
        std::memcpy(accum, tmp.data(), sizeof(int32_t) * tmp.size());
    }
}

/* upstream tLweExtractLweSample: a'_{iN} = a_i[0], a'_{iN+j} = -a_i[N-j],
 * b' = b[0]. */
void orc_extract(const orc_params* P, const int32_t* accum, int32_t* out) {
    const int32_t N = P->N, k = P->k;
    for (int32_t i = 0; i < k; ++i) {
        const int32_t* a = accum + i * N;
        out[i * N] = a[0];
        for (int32_t j = 1; j < N; ++j) out[i * N + j] = wrap_sub(0, a[N - j]);
    }
    out[k * N] = accum[k * N];
}

/* lwe-keyswitch-functions.cpp:228-241 (lweKeySwitch) and :114-129
 * (lweKeySwitchTranslate_fromArray): start from (0, b), subtract
 * KS[i][j][digit] for every non-zero base-2^basebit digit of
 * a_i + 2^(32 - (1 + basebit t)). */
void orc_keyswitch(const orc_params* P, const int32_t* ks, const int32_t* in,
                   int32_t* out) {
    const int32_t n = P->n, n_in = P->k * P->N;
    const int32_t t = P->ks_t, basebit = P->ks_basebit, base = 1 << basebit;
    const uint32_t prec_offset = 1u << (32 - (1 + basebit * t));
    const uint32_t mask = (uint32_t)base - 1;
    std::vector<uint32_t> acc(n + 1, 0);
    acc[n] = (uint32_t)in[n_in];
    for (int32_t i = 0; i < n_in; ++i) {
        const uint32_t aibar = (uint32_t)in[i] + prec_offset;
        for (int32_t j = 0; j < t; ++j) {
            const uint32_t aij = (aibar >> (32 - (j + 1) * basebit)) & mask;
            if (aij == 0) continue;
            const int32_t* row = ks + ((size_t)(i * t + j) * base + aij) * (n + 1);
            for (int32_t q = 0; q <= n; ++q) acc[q] -= (uint32_t)row[q];
        }
    }
    for (int32_t q = 0; q <= n; ++q) out[q] = (int32_t)acc[q];
}

/* tfhe_bootstrap_woKS_FFT.cpp:57-66 (modulus switch, test vector of mu)
 * and mulByXaiOrCopy.cpp:25-41 (X^{2N - barb} rotation, or a copy when
 * barb = 0); the accumulator is the trivial TLWE (0, v). */
void orc_bootstrap_prologue(const orc_params* P, int32_t mu, const int32_t* x,
                            int32_t* bara, int32_t* accum) {
    const int32_t n = P->n, N = P->N, k = P->k;
    const int32_t Nx2 = 2 * N;
    const int32_t barb = orc_mod_switch_from_torus32(x[n], Nx2);
    for (int32_t i = 0; i < n; i++)
        bara[i] = orc_mod_switch_from_torus32(x[i], Nx2);
    std::vector<int32_t> testvect(N, mu);
    std::memset(accum, 0, sizeof(int32_t) * (size_t)k * N);
    if (barb != 0)
        orc_mul_by_xai(N, Nx2 - barb, testvect.data(), accum + k * N);
    else
        std::memcpy(accum + k * N, testvect.data(), sizeof(int32_t) * N);
}

/* Programmable bootstrap (published TFHE algorithm, Chillotti, Joye,
 * Paillier, "Programmable bootstrapping enables efficient homomorphic
 * inference of deep neural networks", 2021): the constant test vector of
 * tfhe_bootstrap_woKS_FFT.cpp:63-66 replaced by an arbitrary polynomial tv;
 * acc = (0, X^{-barb} tv), blind rotation, extraction, key switch. */
void orc_bootstrap_tv(const orc_params* P, const double* bk_fft, const int32_t* ks,
                      const int32_t* tv, const int32_t* x, int32_t* out) {
    const int32_t n = P->n, N = P->N, k = P->k, Nx2 = 2 * N;
    std::vector<int32_t> bara(n), acc((size_t)(k + 1) * N, 0), u((size_t)k * N + 1);
    const int32_t barb = orc_mod_switch_from_torus32(x[n], Nx2);
    for (int32_t i = 0; i < n; i++) bara[i] = orc_mod_switch_from_torus32(x[i], Nx2);
    orc_mul_by_xai(N, (Nx2 - barb) % Nx2, tv, acc.data() + (size_t)k * N);
    orc_blind_rotate_fft(P, acc.data(), bk_fft, bara.data());
    orc_extract(P, acc.data(), u.data());
    orc_keyswitch(P, ks, u.data(), out);
}

void orc_bootstrap_tv_batch(const orc_params* P, const double* bk_fft, const int32_t* ks,
                            const int32_t* tv, int32_t tv_stride, const int32_t* x,
                            int32_t* out, int32_t count, int32_t threads) {
    const int32_t w = P->n + 1;
#pragma omp parallel for schedule(dynamic) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int32_t c = 0; c < count; ++c)
        orc_bootstrap_tv(P, bk_fft, ks, tv + (size_t)c * tv_stride, x + (size_t)c * w,
                         out + (size_t)c * w);
}

/* Test vector of a lookup table on p messages encoded with a padding bit
 * (message m at phase m / (2p)): coefficient j is table[m_j] for the
 * message m_j = floor((j p + N/2) / N) whose window holds j, and -table[0]
 * for the top half-window (j >= N - N/(2p)), which the negacyclic wrap maps
 * back onto message 0 for phases just below 0. */
void orc_test_vector(int32_t N, const int32_t* table, int32_t p, int32_t* tv) {
    for (int32_t j = 0; j < N; ++j) {
        const int64_t m = ((int64_t)j * p + N / 2) / N;
        tv[j] = m < p ? table[m] : (int32_t)(0u - (uint32_t)table[0]);
    }
}

void orc_bootstrap_woks(const orc_params* P, const double* bk_fft, int32_t mu,
                        const int32_t* x, int32_t* out, int32_t exact,
                        const int32_t* bk) {
    std::vector<int32_t> bara(P->n);
    std::vector<int32_t> acc((size_t)(P->k + 1) * P->N);
    orc_bootstrap_prologue(P, mu, x, bara.data(), acc.data());
    if (exact)
        orc_blind_rotate_exact(P, acc.data(), bk, bara.data());
    else
        orc_blind_rotate_fft(P, acc.data(), bk_fft, bara.data());
    orc_extract(P, acc.data(), out);
}

/* Gate linear combinations.  OR is in the reference
 * (tfhe_blindRotate_FFT_tb.cpp:267-276: (0,1/8) + ca + cb); the others
 * restate the upstream boot-gates of the TFHE paper. */
void orc_gate_combine(const orc_params* P, int32_t gate, const int32_t* ca,
                      const int32_t* cb, int32_t* out) {
    const int32_t n = P->n;
    const int32_t e8 = orc_mod_switch_to_torus32(1, 8);
    const int32_t e4 = orc_mod_switch_to_torus32(1, 4);
    int32_t c = 0, sa = 1, sb = 1;
    switch (gate) {
    case ORC_GATE_NAND: c = e8;  sa = -1; sb = -1; break;
    case ORC_GATE_AND:  c = -e8; sa = 1;  sb = 1;  break;
    case ORC_GATE_OR:   c = e8;  sa = 1;  sb = 1;  break;
    case ORC_GATE_XOR:  c = e4;  sa = 2;  sb = 2;  break;
    case ORC_GATE_XNOR: c = -e4; sa = -2; sb = -2; break;
    case ORC_GATE_NOR:  c = -e8; sa = -1; sb = -1; break;
    case ORC_GATE_ANDNY: c = -e8; sa = -1; sb = 1; break;
    case ORC_GATE_ANDYN: c = -e8; sa = 1;  sb = -1; break;
    case ORC_GATE_ORNY: c = e8;  sa = -1; sb = 1;  break;
    case ORC_GATE_ORYN: c = e8;  sa = 1;  sb = -1; break;
    default: c = 0; sa = 0; sb = 0; break;
    }
    for (int32_t i = 0; i <= n; ++i) {
        uint32_t v = (i == n) ? (uint32_t)c : 0u;
        v += (uint32_t)sa * (uint32_t)ca[i];
        v += (uint32_t)sb * (uint32_t)cb[i];
        out[i] = (int32_t)v;
    }
}

void orc_boots_gate(const orc_params* P, const double* bk_fft,
                    const int32_t* ks, int32_t gate, const int32_t* ca,
                    const int32_t* cb, int32_t* out) {
    const int32_t mu = orc_mod_switch_to_torus32(1, 8);
    std::vector<int32_t> tmp(P->n + 1), u((size_t)P->k * P->N + 1);
    orc_gate_combine(P, gate, ca, cb, tmp.data());
    orc_bootstrap_woks(P, bk_fft, mu, tmp.data(), u.data(), 0, nullptr);
    orc_keyswitch(P, ks, u.data(), out);
}

/* upstream bootsMUX: u1 = BS_woKS(AND(a,b)), u2 = BS_woKS(AND(not a, c)),
 * result = KS((0, 1/8) + u1 + u2). */
void orc_boots_mux(const orc_params* P, const double* bk_fft,
                   const int32_t* ks, const int32_t* a, const int32_t* b,
                   const int32_t* c, int32_t* out) {
    const int32_t n = P->n, nk = P->k * P->N;
    const int32_t mu = orc_mod_switch_to_torus32(1, 8);
    std::vector<int32_t> tmp(n + 1), u1(nk + 1), u2(nk + 1), s(nk + 1);
    orc_gate_combine(P, ORC_GATE_AND, a, b, tmp.data());
    orc_bootstrap_woks(P, bk_fft, mu, tmp.data(), u1.data(), 0, nullptr);
    orc_gate_combine(P, ORC_GATE_ANDNY, a, c, tmp.data());
    orc_bootstrap_woks(P, bk_fft, mu, tmp.data(), u2.data(), 0, nullptr);
    for (int32_t i = 0; i <= nk; ++i)
        s[i] = wrap_add(u1[i], u2[i]);
    s[nk] = wrap_add(s[nk], mu);
    orc_keyswitch(P, ks, s.data(), out);
}

/* `count` independent bootsMUX (above) on `threads` OpenMP threads. */
void orc_boots_mux_batch(const orc_params* P, const double* bk_fft,
                         const int32_t* ks, const int32_t* a, const int32_t* b,
                         const int32_t* c, int32_t* out, int32_t count,
                         int32_t threads) {
    const int32_t w = P->n + 1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int32_t g = 0; g < count; ++g)
        orc_boots_mux(P, bk_fft, ks, a + (size_t)g * w, b + (size_t)g * w,
                      c + (size_t)g * w, out + (size_t)g * w);
    (void)threads;
}

void orc_boots_gate_batch(const orc_params* P, const double* bk_fft,
                          const int32_t* ks, const int32_t* gates,
                          const int32_t* ca, const int32_t* cb, int32_t* out,
                          int32_t count, int32_t threads) {
    const int32_t w = P->n + 1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int32_t g = 0; g < count; ++g)
        orc_boots_gate(P, bk_fft, ks, gates[g], ca + (size_t)g * w,
                       cb + (size_t)g * w, out + (size_t)g * w);
    (void)threads;
}

/* `count` independent exact external products: accum (count x (k+1)N) by
 * gsw (count x tgsw words, time domain), on `threads` OpenMP threads. */
void orc_extern_mul_exact_batch(const orc_params* P, int32_t* accum, const int32_t* gsw,
                                int32_t count, int32_t threads) {
    const size_t w_acc = (size_t)(P->k + 1) * P->N;
    const size_t w_gsw = (size_t)(P->k + 1) * P->l * w_acc;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int32_t c = 0; c < count; ++c)
        orc_extern_mul_exact(P, accum + (size_t)c * w_acc, gsw + (size_t)c * w_gsw);
    (void)threads;
}

/* Bootstraps without key switch of `count` samples x (count x (n+1)) into
 * out (count x (kN+1)), exact int64 blind rotation when `exact` (bk in the
 * time domain), else the FFT blind rotation; on `threads` OpenMP threads. */
void orc_bootstrap_woks_batch(const orc_params* P, const double* bk_fft, int32_t mu,
                              const int32_t* x, int32_t* out, int32_t count,
                              int32_t exact, const int32_t* bk, int32_t threads) {
    const int32_t w_in = P->n + 1, w_out = P->k * P->N + 1;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int32_t c = 0; c < count; ++c)
        orc_bootstrap_woks(P, bk_fft, mu, x + (size_t)c * w_in, out + (size_t)c * w_out,
                           exact, bk);
    (void)threads;
}

/* Full gates (combine, bootstrap, key switch) with the exact int64 blind
 * rotation: the exact-product counterpart of orc_boots_gate_batch. */
void orc_boots_gate_exact_batch(const orc_params* P, const int32_t* bk,
                                const int32_t* ks, const int32_t* gates,
                                const int32_t* ca, const int32_t* cb, int32_t* out,
                                int32_t count, int32_t threads) {
    const int32_t w = P->n + 1;
    const int32_t mu = orc_mod_switch_to_torus32(1, 8);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
#endif
    for (int32_t g = 0; g < count; ++g) {
        std::vector<int32_t> tmp(w), u((size_t)P->k * P->N + 1);
        orc_gate_combine(P, gates[g], ca + (size_t)g * w, cb + (size_t)g * w, tmp.data());
        orc_bootstrap_woks(P, nullptr, mu, tmp.data(), u.data(), 1, bk);
        orc_keyswitch(P, ks, u.data(), out + (size_t)g * w);
    }
    (void)threads;
}

int32_t orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
