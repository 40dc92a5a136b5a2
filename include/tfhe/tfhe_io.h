/*
 * tfhe/tfhe_io.h -- the upstream TFHE file calls the reference's test bench
 * uses (test_bench/client/alice.c:19-27,49-54, test_bench/server/cloud.c:
 * 42-56,65-67, test_bench/client/verify.c:8-22), over the engine's own
 * versioned binary format (include/tfhe_keyfile.h).  A file written by one
 * of these functions is read back by its counterpart; the upstream
 * library's files are not readable (its format is not available).
 *
 * The *_fromFile constructors return NULL, after a message on stderr, for a
 * malformed, truncated or corrupted record; the import functions abort in
 * that case (they return nothing, like upstream).
 */
#ifndef TFHE_GB300_COMPAT_TFHE_IO_H
#define TFHE_GB300_COMPAT_TFHE_IO_H

#include <stdio.h>

#include "tfhe.h"

#ifdef __cplusplus
extern "C" {
#endif

void export_tfheGateBootstrappingParameterSet_toFile(FILE* F,
                                                     const TFheGateBootstrappingParameterSet* params);
TFheGateBootstrappingParameterSet* new_tfheGateBootstrappingParameterSet_fromFile(FILE* F);

void export_tfheGateBootstrappingSecretKeySet_toFile(FILE* F,
                                                     const TFheGateBootstrappingSecretKeySet* key);
TFheGateBootstrappingSecretKeySet* new_tfheGateBootstrappingSecretKeySet_fromFile(FILE* F);

void export_tfheGateBootstrappingCloudKeySet_toFile(FILE* F,
                                                    const TFheGateBootstrappingCloudKeySet* bk);
TFheGateBootstrappingCloudKeySet* new_tfheGateBootstrappingCloudKeySet_fromFile(FILE* F);

void export_gate_bootstrapping_ciphertext_toFile(FILE* F, const LweSample* sample,
                                                 const TFheGateBootstrappingParameterSet* params);
void import_gate_bootstrapping_ciphertext_fromFile(FILE* F, LweSample* sample,
                                                   const TFheGateBootstrappingParameterSet* params);

#ifdef __cplusplus
}
#endif
#endif
