/*
 * tfhe/tfhe.h -- the upstream TFHE gate API over the GB300 engine.
 *
 * The reference's test bench (test_bench/client/alice.c,
 * test_bench/server/cloud.c, test_bench/client/verify.c) is written against
 * the upstream TFHE library's <tfhe/tfhe.h> and <tfhe/tfhe_io.h>, which the
 * reference does not vendor.  These two headers give those programs the same
 * call shapes over this engine, so they are recompiled against
 * `-I include` and linked with libtfhe_gb300.so instead of
 * -ltfhe-spqlios-fma (test_bench/Makefile:6).
 *
 * The struct definitions are this engine's own (the upstream layouts are not
 * available); only the members the test bench touches are part of the
 * contract: `bk->params` (cloud.c:46), `key->params` (verify.c:13) and
 * `key->cloud` (alice.c:25).  A ciphertext is an LweSample with its own mask
 * array, created by new_gate_bootstrapping_ciphertext(_array).
 *
 * Gates run on the GPU: the cloud keyset opens an engine context on device 0
 * at its first gate (a client that only encrypts and decrypts never touches
 * the GPU).  Like upstream, the gate functions return nothing; an engine
 * error is printed to stderr and aborts the process (the reference's host
 * exits on device errors too, kernel/src/include/host.h:13-18).
 */
#ifndef TFHE_GB300_COMPAT_TFHE_H
#define TFHE_GB300_COMPAT_TFHE_H

#include <stdint.h>

#include "../tfhe_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t Torus32;

/* One LWE ciphertext: a[n] mask, b body (Torus32), and the noise variance
 * estimate (kept for format compatibility; the engine does not track it). */
typedef struct LweSample {
    Torus32* a;
    Torus32 b;
    double current_variance;
} LweSample;

typedef struct TFheGateBootstrappingParameterSet {
    tfhe_params engine; /* the parameter set in engine form */
} TFheGateBootstrappingParameterSet;

struct tfhe_compat_cloud; /* host keys and the lazily created engine context */

typedef struct TFheGateBootstrappingCloudKeySet {
    const TFheGateBootstrappingParameterSet* params;
    struct tfhe_compat_cloud* impl;
} TFheGateBootstrappingCloudKeySet;

typedef struct TFheGateBootstrappingSecretKeySet {
    const TFheGateBootstrappingParameterSet* params;
    TFheGateBootstrappingCloudKeySet cloud;
    Torus32* lwe_key;  /* n binary coefficients  */
    Torus32* tlwe_key; /* k N binary coefficients */
} TFheGateBootstrappingSecretKeySet;

/* ---- parameters, randomness, keys (alice.c:9-17) ---------------------- */
/* The default gate set (n = 630, N = 1024, k = 1, l = 3, Bgbit = 7, t = 8,
 * basebit = 2; the reference's kernel/src/include/constants.h:26-40) for any
 * minimum_lambda up to 128; NULL above. */
TFheGateBootstrappingParameterSet* new_default_gate_bootstrapping_parameters(int minimum_lambda);
void delete_gate_bootstrapping_parameters(TFheGateBootstrappingParameterSet* params);

/* Seeds the generator of key generation and encryption
 * (numeric-functions.cpp:11-19). */
void tfhe_random_generator_setSeed(uint32_t* values, int32_t size);

TFheGateBootstrappingSecretKeySet* new_random_gate_bootstrapping_secret_keyset(
    const TFheGateBootstrappingParameterSet* params);
void delete_gate_bootstrapping_secret_keyset(TFheGateBootstrappingSecretKeySet* keyset);
void delete_gate_bootstrapping_cloud_keyset(TFheGateBootstrappingCloudKeySet* keyset);

/* ---- ciphertexts ------------------------------------------------------- */
LweSample* new_gate_bootstrapping_ciphertext(const TFheGateBootstrappingParameterSet* params);
LweSample* new_gate_bootstrapping_ciphertext_array(int32_t nbelems,
                                                   const TFheGateBootstrappingParameterSet* params);
void delete_gate_bootstrapping_ciphertext(LweSample* sample);
void delete_gate_bootstrapping_ciphertext_array(int32_t nbelems, LweSample* samples);

/* bootsSymEncrypt / bootsSymDecrypt: bit <-> +-1/8 with the LWE key. */
void bootsSymEncrypt(LweSample* result, int32_t message, const TFheGateBootstrappingSecretKeySet* key);
int32_t bootsSymDecrypt(const LweSample* sample, const TFheGateBootstrappingSecretKeySet* key);

/* ---- gates (cloud.c:10-35) -------------------------------------------- */
void bootsCONSTANT(LweSample* result, int32_t value, const TFheGateBootstrappingCloudKeySet* bk);
void bootsNOT(LweSample* result, const LweSample* ca, const TFheGateBootstrappingCloudKeySet* bk);
void bootsCOPY(LweSample* result, const LweSample* ca, const TFheGateBootstrappingCloudKeySet* bk);
void bootsNAND(LweSample* result, const LweSample* ca, const LweSample* cb,
               const TFheGateBootstrappingCloudKeySet* bk);
void bootsOR(LweSample* result, const LweSample* ca, const LweSample* cb,
             const TFheGateBootstrappingCloudKeySet* bk);
void bootsAND(LweSample* result, const LweSample* ca, const LweSample* cb,
              const TFheGateBootstrappingCloudKeySet* bk);
void bootsXOR(LweSample* result, const LweSample* ca, const LweSample* cb,
              const TFheGateBootstrappingCloudKeySet* bk);
void bootsXNOR(LweSample* result, const LweSample* ca, const LweSample* cb,
               const TFheGateBootstrappingCloudKeySet* bk);
void bootsNOR(LweSample* result, const LweSample* ca, const LweSample* cb,
              const TFheGateBootstrappingCloudKeySet* bk);
void bootsANDNY(LweSample* result, const LweSample* ca, const LweSample* cb,
                const TFheGateBootstrappingCloudKeySet* bk);
void bootsANDYN(LweSample* result, const LweSample* ca, const LweSample* cb,
                const TFheGateBootstrappingCloudKeySet* bk);
void bootsORNY(LweSample* result, const LweSample* ca, const LweSample* cb,
               const TFheGateBootstrappingCloudKeySet* bk);
void bootsORYN(LweSample* result, const LweSample* ca, const LweSample* cb,
               const TFheGateBootstrappingCloudKeySet* bk);
/* result = a ? b : c */
void bootsMUX(LweSample* result, const LweSample* a, const LweSample* b, const LweSample* c,
              const TFheGateBootstrappingCloudKeySet* bk);

/* ---- engine extensions (no upstream counterpart) ----------------------- */
/* Batched forms: `count` independent gates in one GPU batch.  gate is a
 * tfhe_gpu_gate; results[i] = gate(a[i], b[i]). */
void bootsGateArray(int32_t gate, LweSample* results, const LweSample* a, const LweSample* b,
                    int32_t count, const TFheGateBootstrappingCloudKeySet* bk);
void bootsMUXArray(LweSample* results, const LweSample* a, const LweSample* b, const LweSample* c,
                   int32_t count, const TFheGateBootstrappingCloudKeySet* bk);
/* Transform form used by this keyset's gates (default split-FP32). */
void tfhe_gb300_set_form(TFheGateBootstrappingCloudKeySet* bk, tfhe_gpu_form form);
/* The keyset's engine context (opened on first use; NULL if it cannot be). */
tfhe_gpu_ctx* tfhe_gb300_context(const TFheGateBootstrappingCloudKeySet* bk);

#ifdef __cplusplus
}
#endif
#endif
