/*
 * tfhe_keyfile.h -- versioned binary format for keys and ciphertexts, and
 * loading a cloud key file straight into a context's device keys.
 *
 * Replaces the upstream TFHE library's export_*_toFile / *_fromFile calls
 * used by the reference's test bench (test_bench/client/alice.c:19-27,49-54,
 * test_bench/server/cloud.c:42-56,65-67, test_bench/client/verify.c:8-22);
 * that library's own format is not available, so the engine defines its own.
 *
 * A file is a sequence of records.  Every record is a 32-byte header and a
 * payload, all little-endian:
 *
 *   header  0  char[8] magic "TFHEGB3K"
 *           8  u32     format version (TFHE_KEYFILE_VERSION)
 *          12  u32     kind (tfhe_keyfile_kind)
 *          16  u64     payload bytes
 *          24  u32     FNV-1a (32-bit) of the payload
 *          28  u32     zero
 *   payload starts with the parameter block (64 bytes):
 *                      i32 n, N, k, l, Bgbit, ks_t, ks_basebit, split_bits,
 *                      f64 lwe_alpha, tlwe_alpha, 16 zero bytes
 *     PARAMS      nothing more
 *     CLOUD_KEY   u32 bk_domain (0 = time-domain TGSW samples), u32 zero,
 *                 i32 bk[n][(k+1) l][k+1][N], i32 ks[k N][t][2^basebit][n+1]
 *     SECRET_KEY  i32 lwe_key[n], i32 tlwe_key[k N], then the CLOUD_KEY
 *                 payload after its parameter block
 *     CIPHERTEXTS u64 count, i32 samples[count][n+1], f64 variance[count]
 *
 * Readers check the magic, the version, the kind, the payload size against
 * the parameters and the checksum, and return TFHE_GPU_BAD_PARAM with no
 * output written when any check fails.  The bootstrapping key is stored in
 * the time domain (exact integers); loading converts it to the transform
 * forms on the device.
 */
#ifndef TFHE_KEYFILE_H
#define TFHE_KEYFILE_H

#include <stdint.h>
#include <stdio.h>

#include "tfhe_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TFHE_KEYFILE_VERSION 1

typedef enum tfhe_keyfile_kind {
    TFHE_KEYFILE_PARAMS = 1,
    TFHE_KEYFILE_CLOUD_KEY = 2,
    TFHE_KEYFILE_SECRET_KEY = 3,
    TFHE_KEYFILE_CIPHERTEXTS = 4
} tfhe_keyfile_kind;

/* int32 words of the keys of a parameter set. */
int64_t tfhe_keyfile_bk_words(const tfhe_params* params);
int64_t tfhe_keyfile_ks_words(const tfhe_params* params);

/* Next record of a stream: its kind, parameters and item count (samples of
 * a CIPHERTEXTS record, else 1), without consuming it (the stream is left
 * where it was).  Any output may be NULL. */
tfhe_gpu_status tfhe_keyfile_peek(FILE* f, int32_t* kind, tfhe_params* params, int64_t* items);

/* Writers (stream forms; the record is appended at the current position). */
tfhe_gpu_status tfhe_keyfile_write_params(FILE* f, const tfhe_params* params);
tfhe_gpu_status tfhe_keyfile_write_cloud_key(FILE* f, const tfhe_params* params,
                                             const int32_t* bk, const int32_t* ks);
tfhe_gpu_status tfhe_keyfile_write_secret_key(FILE* f, const tfhe_params* params,
                                              const int32_t* lwe_key, const int32_t* tlwe_key,
                                              const int32_t* bk, const int32_t* ks);
/* variance may be NULL (written as zeros). */
tfhe_gpu_status tfhe_keyfile_write_ciphertexts(FILE* f, const tfhe_params* params,
                                               const int32_t* samples, const double* variance,
                                               int64_t count);

/* Readers: consume one record of the given kind.  Output buffers sized by
 * the parameters in the record (tfhe_keyfile_peek first); any buffer may be
 * NULL to skip that part. */
tfhe_gpu_status tfhe_keyfile_read_params(FILE* f, tfhe_params* params);
tfhe_gpu_status tfhe_keyfile_read_cloud_key(FILE* f, tfhe_params* params, int32_t* bk,
                                            int32_t* ks);
tfhe_gpu_status tfhe_keyfile_read_secret_key(FILE* f, tfhe_params* params, int32_t* lwe_key,
                                             int32_t* tlwe_key, int32_t* bk, int32_t* ks);
/* *count: in = capacity of samples (items), out = items read. */
tfhe_gpu_status tfhe_keyfile_read_ciphertexts(FILE* f, tfhe_params* params, int32_t* samples,
                                              double* variance, int64_t* count);

/* Path forms of the whole-file cases. */
tfhe_gpu_status tfhe_keyfile_save_cloud_key(const char* path, const tfhe_params* params,
                                            const int32_t* bk, const int32_t* ks);
tfhe_gpu_status tfhe_keyfile_load_cloud_key(const char* path, tfhe_params* params, int32_t* bk,
                                            int32_t* ks);

/* Read a cloud key record (from a file holding a CLOUD_KEY or SECRET_KEY
 * record) and upload it into the context: the bootstrapping key to the
 * forms in form_mask, and the key-switching key.  The file's parameters
 * must equal the context's (split_bits aside). */
tfhe_gpu_status tfhe_gpu_upload_cloud_key_file(tfhe_gpu_ctx* ctx, const char* path,
                                               uint32_t form_mask);

#ifdef __cplusplus
}
#endif
#endif
