// keygen.cpp -- client side of the engine: key generation, encryption and
// decryption on the host, with the exact RNG and integer semantics of the
// reference's numeric and LWE functions:
//   kernel/src/numeric-functions.cpp:11-76  (engine, distributions, gaussian32,
//                                            dtot32, modSwitch{To,From}Torus32)
//   kernel/src/lwe-functions.cpp:21-93       (lweKeyGen, lweSymEncrypt, lwePhase)
//   kernel/src/lwe-keyswitch-functions.cpp:163-215 (lweCreateKeySwitchKey)
// and of the upstream key-set generation the reference calls
// (new_random_gate_bootstrapping_secret_keyset, alice.c:9-15): LWE key, TLWE
// key, KS key from the extracted TLWE key, then BK_i = TGSW(s_i).
//
// The distributions are the C++ standard library's (std::default_random_engine,
// uniform_int_distribution, normal_distribution), as in the reference, so the
// same seed gives the same keys with the same libstdc++.  A fresh
// normal_distribution per Gaussian sample, as gaussian32 does.
#include <cstring>
#include <limits.h>
#include <random>
#include <vector>

#include "../../include/tfhe_gpu.h"
#include "engine.h"

namespace {

std::default_random_engine g_gen;
std::uniform_int_distribution<int32_t> g_unif(INT32_MIN, INT32_MAX);

inline uint32_t u(int32_t v) { return (uint32_t)v; }

int32_t dtot32(double d) { return (int32_t)(int64_t)((d - (double)(int64_t)d) * 4294967296.0); }

int32_t gaussian32(int32_t message, double sigma) {
    std::normal_distribution<double> distribution(0., sigma);
    const double err = distribution(g_gen);
    return (int32_t)(u(message) + u(dtot32(err)));
}

void lwe_encrypt_noise(int32_t* out, int32_t b, const int32_t* key, int32_t n) {
    uint32_t acc = u(b);
    for (int32_t i = 0; i < n; ++i) {
        out[i] = g_unif(g_gen);
        acc += u(out[i]) * u(key[i]);
    }
    out[n] = (int32_t)acc;
}

// b += key * a (negacyclic, exact; key binary)
void addmul_binary(int32_t N, int32_t* b, const int32_t* key, const int32_t* a) {
    std::vector<uint32_t> acc(N, 0);
    for (int32_t j = 0; j < N; ++j) {
        if (!key[j]) continue;
        const uint32_t kj = u(key[j]);
        for (int32_t i = 0; i < j; ++i) acc[i] -= kj * u(a[i - j + N]);
        for (int32_t i = j; i < N; ++i) acc[i] += kj * u(a[i - j]);
    }
    for (int32_t i = 0; i < N; ++i) b[i] = (int32_t)(u(b[i]) + acc[i]);
}

bool params_ok(const tfhe_params* P) {
    return P && P->n > 0 && P->N > 0 && (P->N & (P->N - 1)) == 0 && P->k >= 1 && P->l >= 1 &&
           P->Bgbit >= 1 && P->l * P->Bgbit <= 32 && P->ks_t >= 1 && P->ks_basebit >= 1 &&
           P->ks_t * P->ks_basebit <= 31;
}

}  // namespace

extern "C" {

void tfhe_client_set_seed(const uint32_t* values, int32_t size) {
    std::seed_seq seeds(values, values + size);
    g_gen.seed(seeds);
}

int32_t tfhe_client_mod_switch_to_torus32(int32_t mu, int32_t Msize) {
    const uint64_t interv = ((UINT64_C(1) << 63) / (uint64_t)Msize) * 2;
    const uint64_t phase64 = (uint64_t)(int64_t)mu * interv;
    return (int32_t)(phase64 >> 32);
}

}  // extern "C"

namespace tfhe_gb300 {

tfhe_gpu_status gate_keyset_host(const tfhe_params* P, int32_t* lwe_key, int32_t* tlwe_key,
                                 int32_t* ks, int32_t* bk, bool bk_products) {
    if (!params_ok(P) || !lwe_key || !tlwe_key || !ks || !bk) return TFHE_GPU_BAD_PARAM;
    const int32_t n = P->n, N = P->N, k = P->k, l = P->l;
    const int32_t kpl = (k + 1) * l;
    // lweKeyGen (lwe-functions.cpp:21-27)
    {
        std::uniform_int_distribution<int32_t> d(0, 1);
        for (int32_t i = 0; i < n; ++i) lwe_key[i] = d(g_gen);
    }
    // tLweKeyGen
    {
        std::uniform_int_distribution<int32_t> d(0, 1);
        for (int32_t i = 0; i < k * N; ++i) tlwe_key[i] = d(g_gen);
    }
    // lweCreateKeySwitchKey (lwe-keyswitch-functions.cpp:163-215), input key
    // = extracted TLWE key (kN bits), output key = LWE key.
    {
        const int32_t n_in = k * N, t = P->ks_t, basebit = P->ks_basebit, base = 1 << basebit;
        const int32_t sizeks = n_in * t * (base - 1);
        std::vector<double> noise(sizeks);
        double err = 0;
        for (int32_t i = 0; i < sizeks; ++i) {
            std::normal_distribution<double> d(0., P->lwe_alpha);
            noise[i] = d(g_gen);
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
                    const uint32_t mess = u(tlwe_key[i]) * (uint32_t)h * (1u << (32 - (j + 1) * basebit));
                    lwe_encrypt_noise(row0 + (size_t)h * (n + 1),
                                      (int32_t)(mess + u(dtot32(noise[index]))), lwe_key, n);
                    ++index;
                }
            }
    }
    // BK_i = tGswSymEncryptInt(s_i): kpl TLWE encryptions of zero, then
    // s_i h_j added to coefficient 0 of polynomial i of row (i, j).
    {
        const size_t tgsw = (size_t)kpl * (k + 1) * N;
        for (int32_t s = 0; s < n; ++s) {
            int32_t* g = bk + s * tgsw;
            for (int32_t p = 0; p < kpl; ++p) {
                int32_t* row = g + (size_t)p * (k + 1) * N;
                int32_t* b = row + (size_t)k * N;
                for (int32_t j = 0; j < N; ++j) b[j] = gaussian32(0, P->tlwe_alpha);
                for (int32_t i = 0; i < k; ++i) {
                    int32_t* a = row + (size_t)i * N;
                    for (int32_t j = 0; j < N; ++j) a[j] = g_unif(g_gen);
                    if (bk_products) addmul_binary(N, b, tlwe_key + i * N, a);
                }
            }
            if (!bk_products) continue;  // finished on the device (launch_tgsw_finish)
            for (int32_t i = 0; i <= k; ++i)
                for (int32_t j = 0; j < l; ++j) {
                    int32_t* row = g + (size_t)(i * l + j) * (k + 1) * N;
                    const uint32_t h = 1u << (32 - (j + 1) * P->Bgbit);
                    row[i * N] = (int32_t)(u(row[i * N]) + u(lwe_key[s]) * h);
                }
        }
    }
    return TFHE_GPU_OK;
}

}  // namespace tfhe_gb300

extern "C" {

tfhe_gpu_status tfhe_client_gate_keyset(const tfhe_params* P, int32_t* lwe_key,
                                        int32_t* tlwe_key, int32_t* ks, int32_t* bk) {
    return tfhe_gb300::gate_keyset_host(P, lwe_key, tlwe_key, ks, bk, true);
}

tfhe_gpu_status tfhe_client_test_vector(int32_t N, const int32_t* table, int32_t p, int32_t* tv) {
    if (N <= 0 || p <= 0 || p > N || !table || !tv) return TFHE_GPU_BAD_PARAM;
    // coefficient j belongs to the message whose phase window m/(2p) +-
    // 1/(4p) holds j/(2N); the top half-window wraps (negacyclically) onto
    // message 0 from below, hence -table[0] there
    for (int32_t j = 0; j < N; ++j) {
        const int64_t m = ((int64_t)j * p + N / 2) / N;
        tv[j] = m < p ? table[m] : (int32_t)(0u - (uint32_t)table[0]);
    }
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_client_encrypt_phases(const tfhe_params* P, const int32_t* mu,
                                           int32_t count, const int32_t* lwe_key, int32_t* out) {
    if (!params_ok(P) || count < 0 || (count && (!mu || !lwe_key || !out))) return TFHE_GPU_BAD_PARAM;
    for (int32_t c = 0; c < count; ++c)
        lwe_encrypt_noise(out + (size_t)c * (P->n + 1), gaussian32(mu[c], P->lwe_alpha), lwe_key, P->n);
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_client_encrypt_bits(const tfhe_params* P, const int32_t* bits,
                                         int32_t count, const int32_t* lwe_key, int32_t* out) {
    if (!params_ok(P) || count < 0 || (count && (!bits || !lwe_key || !out)))
        return TFHE_GPU_BAD_PARAM;
    const int32_t s8 = tfhe_client_mod_switch_to_torus32(1, 8);
    for (int32_t c = 0; c < count; ++c) {
        const int32_t mu = bits[c] ? s8 : -s8;
        lwe_encrypt_noise(out + (size_t)c * (P->n + 1), gaussian32(mu, P->lwe_alpha), lwe_key, P->n);
    }
    return TFHE_GPU_OK;
}

void tfhe_client_phases(const int32_t* samples, int32_t count, int32_t dim, const int32_t* key,
                        int32_t* phases) {
    for (int32_t c = 0; c < count; ++c) {
        const int32_t* s = samples + (size_t)c * (dim + 1);
        uint32_t axs = 0;
        for (int32_t i = 0; i < dim; ++i) axs += u(s[i]) * u(key[i]);
        phases[c] = (int32_t)(u(s[dim]) - axs);
    }
}

tfhe_gpu_status tfhe_client_decrypt_bits(const tfhe_params* P, const int32_t* samples,
                                         int32_t count, const int32_t* lwe_key, int32_t* bits) {
    if (!params_ok(P) || count < 0 || (count && (!samples || !lwe_key || !bits)))
        return TFHE_GPU_BAD_PARAM;
    std::vector<int32_t> ph(count > 0 ? count : 1);
    tfhe_client_phases(samples, count, P->n, lwe_key, ph.data());
    for (int32_t c = 0; c < count; ++c) bits[c] = ph[c] > 0 ? 1 : 0;
    return TFHE_GPU_OK;
}

}  // extern "C"
