// compat.cpp -- the upstream TFHE gate and file API (include/tfhe/tfhe.h,
// include/tfhe/tfhe_io.h) over the engine's C ABI, so the reference's test
// bench programs (test_bench/client/alice.c, test_bench/server/cloud.c,
// test_bench/client/verify.c) recompile against this library unchanged.
//
// Keys are held on the host in the time domain (for export) and uploaded to
// an engine context on device 0 at the first gate.  Gates copy their input
// samples into one contiguous host batch, run the engine's host-buffer entry
// points and copy the results out, so a result may alias an input (cloud.c
// does this at :21 and :12).
//
// With the environment variable TFHE_GB300_TRACE set (to anything), every
// gate call prints one line to stderr: the call, its batch size, the device
// it ran on and its host-side time.  It lets a user of an unmodified program
// see that its gates ran on the GPU.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/tfhe/tfhe.h"
#include "../../include/tfhe/tfhe_io.h"
#include "../../include/tfhe_gpu.h"
#include "../../include/tfhe_keyfile.h"

struct tfhe_compat_cloud {
    TFheGateBootstrappingParameterSet* owned_params = nullptr;  // set when read from a file
    std::vector<int32_t> bk, ks;  // time-domain keys
    std::mutex mu;
    tfhe_gpu_ctx* ctx = nullptr;
    bool ctx_failed = false;
    tfhe_gpu_form form = TFHE_GPU_SPLIT_FP32;
    uint32_t uploaded = 0;  // form mask of the bootstrapping keys on the device
    std::vector<int32_t> in0, in1, in2, out;
};

namespace {

[[noreturn]] void die(const char* fn, const char* what) {
    std::fprintf(stderr, "tfhe_gb300: %s: %s\n", fn, what);
    std::fflush(stderr);
    std::abort();
}

int32_t mu8() { return tfhe_client_mod_switch_to_torus32(1, 8); }

int32_t dim(const TFheGateBootstrappingParameterSet* p) { return p->engine.n; }

TFheGateBootstrappingParameterSet* new_params(const tfhe_params& P) {
    auto* p = new TFheGateBootstrappingParameterSet;
    p->engine = P;
    return p;
}

void pack(std::vector<int32_t>& dst, const LweSample* s, int32_t count, int32_t n) {
    dst.resize((size_t)count * (n + 1));
    for (int32_t c = 0; c < count; ++c) {
        std::memcpy(&dst[(size_t)c * (n + 1)], s[c].a, sizeof(int32_t) * n);
        dst[(size_t)c * (n + 1) + n] = s[c].b;
    }
}

void unpack(LweSample* s, const std::vector<int32_t>& src, int32_t count, int32_t n) {
    for (int32_t c = 0; c < count; ++c) {
        std::memcpy(s[c].a, &src[(size_t)c * (n + 1)], sizeof(int32_t) * n);
        s[c].b = src[(size_t)c * (n + 1) + n];
        s[c].current_variance = 0.0;
    }
}

// The keyset's engine context with the bootstrapping key of the current form
// on the device; opened and filled on first use.  Caller holds impl->mu.
tfhe_gpu_ctx* ready_ctx(const TFheGateBootstrappingCloudKeySet* bk, const char* fn) {
    if (!bk || !bk->impl || !bk->params) die(fn, "null cloud keyset");
    tfhe_compat_cloud* I = bk->impl;
    if (I->ctx_failed) die(fn, "the engine context could not be opened");
    tfhe_gpu_status s = TFHE_GPU_OK;
    if (!I->ctx) {
        s = tfhe_gpu_create(&bk->params->engine, 0, &I->ctx);
        if (s != TFHE_GPU_OK) {
            I->ctx_failed = true;
            die(fn, tfhe_gpu_status_string(s));
        }
        s = tfhe_gpu_upload_keyswitch_key(I->ctx, I->ks.data());
        if (s != TFHE_GPU_OK) die(fn, tfhe_gpu_last_error(I->ctx));
    }
    const uint32_t m = TFHE_GPU_FORM_MASK(I->form);
    if (!(I->uploaded & m)) {
        s = tfhe_gpu_upload_bootstrapping_key(I->ctx, I->bk.data(), m);
        if (s != TFHE_GPU_OK) die(fn, tfhe_gpu_last_error(I->ctx));
        I->uploaded |= m;
    }
    return I->ctx;
}

bool tracing() {
    static const bool on = std::getenv("TFHE_GB300_TRACE") != nullptr;
    return on;
}

const char* form_name(tfhe_gpu_form f) { return f == TFHE_GPU_FP64 ? "fp64" : "split_fp32"; }

// one trace line per call (TFHE_GB300_TRACE)
void trace(const char* fn, int32_t count, tfhe_gpu_form form,
           std::chrono::steady_clock::time_point t0) {
    const double ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int dev = -1;
    cudaDeviceProp prop{};
    const bool ok = cudaGetDevice(&dev) == cudaSuccess &&
                    cudaGetDeviceProperties(&prop, dev) == cudaSuccess;
    std::fprintf(stderr, "tfhe_gb300 trace: %s: %d sample(s) on GPU %d (%s, sm_%d%d), %s form, %.3f ms\n",
                 fn, count, dev, ok ? prop.name : "?", ok ? prop.major : 0, ok ? prop.minor : 0,
                 form_name(form), ms);
}

void gate_batch(const char* fn, int32_t gate, LweSample* res, const LweSample* a, const LweSample* b,
                int32_t count, const TFheGateBootstrappingCloudKeySet* bk) {
    if (count <= 0) return;
    const auto t0 = std::chrono::steady_clock::now();
    if (!res || !a || !b) die(fn, "null sample");
    if (!bk || !bk->impl) die(fn, "null cloud keyset");
    std::lock_guard<std::mutex> lock(bk->impl->mu);
    tfhe_gpu_ctx* ctx = ready_ctx(bk, fn);
    tfhe_compat_cloud* I = bk->impl;
    const int32_t n = dim(bk->params);
    pack(I->in0, a, count, n);
    pack(I->in1, b, count, n);
    I->out.resize((size_t)count * (n + 1));
    const tfhe_gpu_status s = tfhe_gpu_bootsGates_host(ctx, nullptr, gate, I->out.data(), I->in0.data(),
                                                       I->in1.data(), count, I->form);
    if (s != TFHE_GPU_OK) die(fn, tfhe_gpu_last_error(ctx));
    unpack(res, I->out, count, n);
    if (tracing()) trace(fn, count, I->form, t0);
}

void mux_batch(const char* fn, LweSample* res, const LweSample* a, const LweSample* b,
               const LweSample* c, int32_t count, const TFheGateBootstrappingCloudKeySet* bk) {
    if (count <= 0) return;
    const auto t0 = std::chrono::steady_clock::now();
    if (!res || !a || !b || !c) die(fn, "null sample");
    if (!bk || !bk->impl) die(fn, "null cloud keyset");
    std::lock_guard<std::mutex> lock(bk->impl->mu);
    tfhe_gpu_ctx* ctx = ready_ctx(bk, fn);
    tfhe_compat_cloud* I = bk->impl;
    const int32_t n = dim(bk->params);
    pack(I->in0, a, count, n);
    pack(I->in1, b, count, n);
    pack(I->in2, c, count, n);
    I->out.resize((size_t)count * (n + 1));
    const tfhe_gpu_status s = tfhe_gpu_bootsMUX_host(ctx, I->out.data(), I->in0.data(), I->in1.data(),
                                                     I->in2.data(), count, I->form);
    if (s != TFHE_GPU_OK) die(fn, tfhe_gpu_last_error(ctx));
    unpack(res, I->out, count, n);
    if (tracing()) trace(fn, count, I->form, t0);
}

void free_impl(tfhe_compat_cloud* I) {
    if (!I) return;
    if (I->ctx) tfhe_gpu_destroy(I->ctx);
    delete I->owned_params;
    delete I;
}

}  // namespace

extern "C" {

// ---- parameters, randomness, keys ---------------------------------------

TFheGateBootstrappingParameterSet* new_default_gate_bootstrapping_parameters(int minimum_lambda) {
    if (minimum_lambda > 128) {
        std::fprintf(stderr, "tfhe_gb300: no parameter set above 128 bits of security\n");
        return nullptr;
    }
    tfhe_params P;
    tfhe_gpu_default_params(&P);
    return new_params(P);
}

void delete_gate_bootstrapping_parameters(TFheGateBootstrappingParameterSet* params) { delete params; }

void tfhe_random_generator_setSeed(uint32_t* values, int32_t size) {
    tfhe_client_set_seed(values, size);
}

TFheGateBootstrappingSecretKeySet* new_random_gate_bootstrapping_secret_keyset(
    const TFheGateBootstrappingParameterSet* params) {
    if (!params) return nullptr;
    const tfhe_params& P = params->engine;
    auto* key = new TFheGateBootstrappingSecretKeySet;
    auto* I = new tfhe_compat_cloud;
    key->params = params;
    key->cloud.params = params;
    key->cloud.impl = I;
    key->lwe_key = new Torus32[P.n];
    key->tlwe_key = new Torus32[(size_t)P.k * P.N];
    I->bk.resize((size_t)tfhe_keyfile_bk_words(&P));
    I->ks.resize((size_t)tfhe_keyfile_ks_words(&P));
    if (tfhe_client_gate_keyset(&P, key->lwe_key, key->tlwe_key, I->ks.data(), I->bk.data()) !=
        TFHE_GPU_OK) {
        delete_gate_bootstrapping_secret_keyset(key);
        return nullptr;
    }
    return key;
}

void delete_gate_bootstrapping_secret_keyset(TFheGateBootstrappingSecretKeySet* key) {
    if (!key) return;
    free_impl(key->cloud.impl);
    delete[] key->lwe_key;
    delete[] key->tlwe_key;
    delete key;
}

void delete_gate_bootstrapping_cloud_keyset(TFheGateBootstrappingCloudKeySet* bk) {
    if (!bk) return;
    free_impl(bk->impl);
    delete bk;
}

// ---- ciphertexts ---------------------------------------------------------

LweSample* new_gate_bootstrapping_ciphertext(const TFheGateBootstrappingParameterSet* params) {
    return new_gate_bootstrapping_ciphertext_array(1, params);
}

LweSample* new_gate_bootstrapping_ciphertext_array(int32_t nbelems,
                                                   const TFheGateBootstrappingParameterSet* params) {
    if (!params || nbelems < 0) return nullptr;
    const int32_t n = dim(params);
    auto* s = new LweSample[nbelems > 0 ? nbelems : 1];
    for (int32_t i = 0; i < nbelems; ++i) {
        s[i].a = new Torus32[n]();
        s[i].b = 0;
        s[i].current_variance = 0.0;
    }
    return s;
}

void delete_gate_bootstrapping_ciphertext(LweSample* sample) {
    delete_gate_bootstrapping_ciphertext_array(1, sample);
}

void delete_gate_bootstrapping_ciphertext_array(int32_t nbelems, LweSample* samples) {
    if (!samples) return;
    for (int32_t i = 0; i < nbelems; ++i) delete[] samples[i].a;
    delete[] samples;
}

void bootsSymEncrypt(LweSample* result, int32_t message, const TFheGateBootstrappingSecretKeySet* key) {
    if (!result || !key) die("bootsSymEncrypt", "null argument");
    const tfhe_params& P = key->params->engine;
    std::vector<int32_t> buf((size_t)P.n + 1);
    const int32_t bit = message ? 1 : 0;
    if (tfhe_client_encrypt_bits(&P, &bit, 1, key->lwe_key, buf.data()) != TFHE_GPU_OK)
        die("bootsSymEncrypt", "encryption failed");
    unpack(result, buf, 1, P.n);
    result->current_variance = P.lwe_alpha * P.lwe_alpha;
}

int32_t bootsSymDecrypt(const LweSample* sample, const TFheGateBootstrappingSecretKeySet* key) {
    if (!sample || !key) die("bootsSymDecrypt", "null argument");
    const tfhe_params& P = key->params->engine;
    std::vector<int32_t> buf;
    pack(buf, sample, 1, P.n);
    int32_t bit = 0;
    if (tfhe_client_decrypt_bits(&P, buf.data(), 1, key->lwe_key, &bit) != TFHE_GPU_OK)
        die("bootsSymDecrypt", "decryption failed");
    return bit;
}

// ---- gates ---------------------------------------------------------------

void bootsCONSTANT(LweSample* result, int32_t value, const TFheGateBootstrappingCloudKeySet* bk) {
    if (!result || !bk) die("bootsCONSTANT", "null argument");
    std::memset(result->a, 0, sizeof(int32_t) * dim(bk->params));
    result->b = value ? mu8() : -mu8();
    result->current_variance = 0.0;
}

void bootsNOT(LweSample* result, const LweSample* ca, const TFheGateBootstrappingCloudKeySet* bk) {
    if (!result || !ca || !bk) die("bootsNOT", "null argument");
    const int32_t n = dim(bk->params);
    for (int32_t i = 0; i < n; ++i) result->a[i] = (int32_t)(0u - (uint32_t)ca->a[i]);
    result->b = (int32_t)(0u - (uint32_t)ca->b);
    result->current_variance = ca->current_variance;
}

void bootsCOPY(LweSample* result, const LweSample* ca, const TFheGateBootstrappingCloudKeySet* bk) {
    if (!result || !ca || !bk) die("bootsCOPY", "null argument");
    if (result != ca) std::memmove(result->a, ca->a, sizeof(int32_t) * dim(bk->params));
    result->b = ca->b;
    result->current_variance = ca->current_variance;
}

#define TFHE_GB300_GATE(NAME, ID)                                                         \
    void NAME(LweSample* result, const LweSample* ca, const LweSample* cb,                \
              const TFheGateBootstrappingCloudKeySet* bk) {                               \
        gate_batch(#NAME, ID, result, ca, cb, 1, bk);                                     \
    }
TFHE_GB300_GATE(bootsNAND, TFHE_GATE_NAND)
TFHE_GB300_GATE(bootsAND, TFHE_GATE_AND)
TFHE_GB300_GATE(bootsOR, TFHE_GATE_OR)
TFHE_GB300_GATE(bootsXOR, TFHE_GATE_XOR)
TFHE_GB300_GATE(bootsXNOR, TFHE_GATE_XNOR)
TFHE_GB300_GATE(bootsNOR, TFHE_GATE_NOR)
TFHE_GB300_GATE(bootsANDNY, TFHE_GATE_ANDNY)
TFHE_GB300_GATE(bootsANDYN, TFHE_GATE_ANDYN)
TFHE_GB300_GATE(bootsORNY, TFHE_GATE_ORNY)
TFHE_GB300_GATE(bootsORYN, TFHE_GATE_ORYN)
#undef TFHE_GB300_GATE

void bootsMUX(LweSample* result, const LweSample* a, const LweSample* b, const LweSample* c,
              const TFheGateBootstrappingCloudKeySet* bk) {
    mux_batch("bootsMUX", result, a, b, c, 1, bk);
}

void bootsGateArray(int32_t gate, LweSample* results, const LweSample* a, const LweSample* b,
                    int32_t count, const TFheGateBootstrappingCloudKeySet* bk) {
    if (gate < TFHE_GATE_NAND || gate > TFHE_GATE_ORYN) die("bootsGateArray", "unknown gate");
    gate_batch("bootsGateArray", gate, results, a, b, count, bk);
}

void bootsMUXArray(LweSample* results, const LweSample* a, const LweSample* b, const LweSample* c,
                   int32_t count, const TFheGateBootstrappingCloudKeySet* bk) {
    mux_batch("bootsMUXArray", results, a, b, c, count, bk);
}

void tfhe_gb300_set_form(TFheGateBootstrappingCloudKeySet* bk, tfhe_gpu_form form) {
    if (!bk || !bk->impl) die("tfhe_gb300_set_form", "null cloud keyset");
    if (form != TFHE_GPU_FP64 && form != TFHE_GPU_SPLIT_FP32) die("tfhe_gb300_set_form", "unknown form");
    std::lock_guard<std::mutex> lock(bk->impl->mu);
    bk->impl->form = form;
}

tfhe_gpu_ctx* tfhe_gb300_context(const TFheGateBootstrappingCloudKeySet* bk) {
    if (!bk || !bk->impl) return nullptr;
    std::lock_guard<std::mutex> lock(bk->impl->mu);
    return ready_ctx(bk, "tfhe_gb300_context");
}

// ---- files ---------------------------------------------------------------

void export_tfheGateBootstrappingParameterSet_toFile(FILE* F,
                                                     const TFheGateBootstrappingParameterSet* params) {
    if (!params || tfhe_keyfile_write_params(F, &params->engine) != TFHE_GPU_OK)
        die("export_tfheGateBootstrappingParameterSet_toFile", "write failed");
}

TFheGateBootstrappingParameterSet* new_tfheGateBootstrappingParameterSet_fromFile(FILE* F) {
    tfhe_params P;
    if (!F || tfhe_keyfile_read_params(F, &P) != TFHE_GPU_OK) {
        std::fprintf(stderr, "tfhe_gb300: not a parameter-set record\n");
        return nullptr;
    }
    return new_params(P);
}

void export_tfheGateBootstrappingSecretKeySet_toFile(FILE* F, const TFheGateBootstrappingSecretKeySet* key) {
    if (!key || !key->cloud.impl ||
        tfhe_keyfile_write_secret_key(F, &key->params->engine, key->lwe_key, key->tlwe_key,
                                      key->cloud.impl->bk.data(), key->cloud.impl->ks.data()) != TFHE_GPU_OK)
        die("export_tfheGateBootstrappingSecretKeySet_toFile", "write failed");
}

TFheGateBootstrappingSecretKeySet* new_tfheGateBootstrappingSecretKeySet_fromFile(FILE* F) {
    int32_t kind = 0;
    tfhe_params P;
    if (!F || tfhe_keyfile_peek(F, &kind, &P, nullptr) != TFHE_GPU_OK || kind != TFHE_KEYFILE_SECRET_KEY) {
        std::fprintf(stderr, "tfhe_gb300: not a secret-key record\n");
        return nullptr;
    }
    auto* I = new tfhe_compat_cloud;
    I->owned_params = new_params(P);
    I->bk.resize((size_t)tfhe_keyfile_bk_words(&P));
    I->ks.resize((size_t)tfhe_keyfile_ks_words(&P));
    auto* key = new TFheGateBootstrappingSecretKeySet;
    key->params = I->owned_params;
    key->cloud.params = I->owned_params;
    key->cloud.impl = I;
    key->lwe_key = new Torus32[P.n];
    key->tlwe_key = new Torus32[(size_t)P.k * P.N];
    if (tfhe_keyfile_read_secret_key(F, nullptr, key->lwe_key, key->tlwe_key, I->bk.data(),
                                     I->ks.data()) != TFHE_GPU_OK) {
        std::fprintf(stderr, "tfhe_gb300: corrupted secret-key record\n");
        delete_gate_bootstrapping_secret_keyset(key);
        return nullptr;
    }
    return key;
}

void export_tfheGateBootstrappingCloudKeySet_toFile(FILE* F, const TFheGateBootstrappingCloudKeySet* bk) {
    if (!bk || !bk->impl ||
        tfhe_keyfile_write_cloud_key(F, &bk->params->engine, bk->impl->bk.data(), bk->impl->ks.data()) !=
            TFHE_GPU_OK)
        die("export_tfheGateBootstrappingCloudKeySet_toFile", "write failed");
}

TFheGateBootstrappingCloudKeySet* new_tfheGateBootstrappingCloudKeySet_fromFile(FILE* F) {
    int32_t kind = 0;
    tfhe_params P;
    if (!F || tfhe_keyfile_peek(F, &kind, &P, nullptr) != TFHE_GPU_OK || kind != TFHE_KEYFILE_CLOUD_KEY) {
        std::fprintf(stderr, "tfhe_gb300: not a cloud-key record\n");
        return nullptr;
    }
    auto* I = new tfhe_compat_cloud;
    I->owned_params = new_params(P);
    I->bk.resize((size_t)tfhe_keyfile_bk_words(&P));
    I->ks.resize((size_t)tfhe_keyfile_ks_words(&P));
    if (tfhe_keyfile_read_cloud_key(F, nullptr, I->bk.data(), I->ks.data()) != TFHE_GPU_OK) {
        std::fprintf(stderr, "tfhe_gb300: corrupted cloud-key record\n");
        free_impl(I);
        return nullptr;
    }
    auto* bk = new TFheGateBootstrappingCloudKeySet;
    bk->params = I->owned_params;
    bk->impl = I;
    return bk;
}

void export_gate_bootstrapping_ciphertext_toFile(FILE* F, const LweSample* sample,
                                                 const TFheGateBootstrappingParameterSet* params) {
    if (!sample || !params) die("export_gate_bootstrapping_ciphertext_toFile", "null argument");
    std::vector<int32_t> buf;
    pack(buf, sample, 1, dim(params));
    if (tfhe_keyfile_write_ciphertexts(F, &params->engine, buf.data(), &sample->current_variance, 1) !=
        TFHE_GPU_OK)
        die("export_gate_bootstrapping_ciphertext_toFile", "write failed");
}

void import_gate_bootstrapping_ciphertext_fromFile(FILE* F, LweSample* sample,
                                                   const TFheGateBootstrappingParameterSet* params) {
    if (!sample || !params) die("import_gate_bootstrapping_ciphertext_fromFile", "null argument");
    const int32_t n = dim(params);
    std::vector<int32_t> buf((size_t)n + 1);
    double var = 0;
    int64_t count = 1;
    tfhe_params P;
    if (!F || tfhe_keyfile_read_ciphertexts(F, &P, buf.data(), &var, &count) != TFHE_GPU_OK || count != 1 ||
        P.n != n)
        die("import_gate_bootstrapping_ciphertext_fromFile", "not a matching ciphertext record");
    unpack(sample, buf, 1, n);
    sample->current_variance = var;
}

}  // extern "C"
