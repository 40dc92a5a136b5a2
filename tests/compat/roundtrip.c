/*
 * roundtrip.c -- a client / cloud / verifier round trip written against the
 * upstream TFHE API as provided by include/tfhe/tfhe.h and tfhe_io.h over the
 * GB300 engine.  Same flow as the reference's test bench (alice.c generates
 * keys and encrypts, cloud.c computes on ciphertexts read from files,
 * verify.c decrypts), in one program with every step going through files in
 * the directory given as argv[1].
 *
 * The cloud computes, on two encrypted 16-bit words x and y:
 *   OR, AND, XOR, NAND, NOR, XNOR, ANDNY, ANDYN, ORNY, ORYN (bitwise, one
 *   gate call per bit), NOT x, a copy of y, the constant 0x5A5A, the smaller
 *   of x and y (an XNOR + MUX comparator chain and a MUX select), and x + y
 *   by a ripple-carry adder, plus one batched bootsGateArray and
 *   bootsMUXArray call; the verifier checks each against the plaintext.
 * Exit status 0 when every result decrypts correctly.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <tfhe/tfhe.h>
#include <tfhe/tfhe_io.h>

#define BITS 16

static char path_buf[4096];
static const char* in_dir(const char* dir, const char* name) {
    snprintf(path_buf, sizeof(path_buf), "%s/%s", dir, name);
    return path_buf;
}

static FILE* open_or_die(const char* path, const char* mode) {
    FILE* f = fopen(path, mode);
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path);
        exit(2);
    }
    return f;
}

/* result = (a == b) ? carry : a, bit by bit from the least significant:
 * at the end carry = 1 when y < x ("take y"). */
static void smaller(LweSample* out, const LweSample* x, const LweSample* y, int nb,
                    const TFheGateBootstrappingCloudKeySet* bk) {
    const TFheGateBootstrappingParameterSet* params = bk->params;
    LweSample* t = new_gate_bootstrapping_ciphertext_array(2, params);
    bootsCONSTANT(&t[0], 0, bk);
    for (int i = 0; i < nb; ++i) {
        bootsXNOR(&t[1], &x[i], &y[i], bk);
        bootsMUX(&t[0], &t[1], &t[0], &x[i], bk); /* equal: keep; else take x_i */
    }
    /* t[0] = 1 when x > y at the most significant differing bit */
    for (int i = 0; i < nb; ++i) bootsMUX(&out[i], &t[0], &y[i], &x[i], bk);
    delete_gate_bootstrapping_ciphertext_array(2, t);
}

static void adder(LweSample* out, const LweSample* x, const LweSample* y, int nb,
                  const TFheGateBootstrappingCloudKeySet* bk) {
    const TFheGateBootstrappingParameterSet* params = bk->params;
    LweSample* t = new_gate_bootstrapping_ciphertext_array(4, params);
    bootsCONSTANT(&t[0], 0, bk); /* carry */
    for (int i = 0; i < nb; ++i) {
        bootsXOR(&t[1], &x[i], &y[i], bk);
        bootsXOR(&out[i], &t[1], &t[0], bk);
        bootsAND(&t[2], &x[i], &y[i], bk);
        bootsAND(&t[3], &t[1], &t[0], bk);
        bootsOR(&t[0], &t[2], &t[3], bk);
    }
    delete_gate_bootstrapping_ciphertext_array(4, t);
}

typedef void (*gate2)(LweSample*, const LweSample*, const LweSample*,
                      const TFheGateBootstrappingCloudKeySet*);

static int client(const char* dir, uint16_t x, uint16_t y) {
    TFheGateBootstrappingParameterSet* params = new_default_gate_bootstrapping_parameters(110);
    uint32_t seed[] = {27, 18, 28};
    tfhe_random_generator_setSeed(seed, 3);
    TFheGateBootstrappingSecretKeySet* key = new_random_gate_bootstrapping_secret_keyset(params);
    FILE* f = open_or_die(in_dir(dir, "secret.key"), "wb");
    export_tfheGateBootstrappingSecretKeySet_toFile(f, key);
    fclose(f);
    f = open_or_die(in_dir(dir, "cloud.key"), "wb");
    export_tfheGateBootstrappingCloudKeySet_toFile(f, &key->cloud);
    fclose(f);
    LweSample* c = new_gate_bootstrapping_ciphertext_array(2 * BITS, params);
    for (int i = 0; i < BITS; ++i) bootsSymEncrypt(&c[i], (x >> i) & 1, key);
    for (int i = 0; i < BITS; ++i) bootsSymEncrypt(&c[BITS + i], (y >> i) & 1, key);
    f = open_or_die(in_dir(dir, "cloud.data"), "wb");
    for (int i = 0; i < 2 * BITS; ++i) export_gate_bootstrapping_ciphertext_toFile(f, &c[i], params);
    fclose(f);
    delete_gate_bootstrapping_ciphertext_array(2 * BITS, c);
    delete_gate_bootstrapping_secret_keyset(key);
    delete_gate_bootstrapping_parameters(params);
    return 0;
}

#define NRES 18

static int cloud(const char* dir) {
    FILE* f = open_or_die(in_dir(dir, "cloud.key"), "rb");
    TFheGateBootstrappingCloudKeySet* bk = new_tfheGateBootstrappingCloudKeySet_fromFile(f);
    fclose(f);
    if (!bk) return 3;
    const TFheGateBootstrappingParameterSet* params = bk->params;
    LweSample* x = new_gate_bootstrapping_ciphertext_array(BITS, params);
    LweSample* y = new_gate_bootstrapping_ciphertext_array(BITS, params);
    f = open_or_die(in_dir(dir, "cloud.data"), "rb");
    for (int i = 0; i < BITS; ++i) import_gate_bootstrapping_ciphertext_fromFile(f, &x[i], params);
    for (int i = 0; i < BITS; ++i) import_gate_bootstrapping_ciphertext_fromFile(f, &y[i], params);
    fclose(f);

    LweSample* r = new_gate_bootstrapping_ciphertext_array(NRES * BITS, params);
    gate2 gates[10] = {bootsOR, bootsAND, bootsXOR, bootsNAND, bootsNOR,
                       bootsXNOR, bootsANDNY, bootsANDYN, bootsORNY, bootsORYN};
    for (int g = 0; g < 10; ++g)
        for (int i = 0; i < BITS; ++i) gates[g](&r[g * BITS + i], &x[i], &y[i], bk);
    for (int i = 0; i < BITS; ++i) bootsNOT(&r[10 * BITS + i], &x[i], bk);
    for (int i = 0; i < BITS; ++i) bootsCOPY(&r[11 * BITS + i], &y[i], bk);
    for (int i = 0; i < BITS; ++i) bootsCONSTANT(&r[12 * BITS + i], (0x5A5A >> i) & 1, bk);
    smaller(&r[13 * BITS], x, y, BITS, bk);
    adder(&r[14 * BITS], x, y, BITS, bk);
    /* batched forms: XOR of all bits at once; MUX(x, y, NOT x) */
    bootsGateArray(TFHE_GATE_XOR, &r[15 * BITS], x, y, BITS, bk);
    bootsMUXArray(&r[16 * BITS], x, y, &r[10 * BITS], BITS, bk);
    /* a result may alias an input: y' = y AND x, written over a copy of y */
    for (int i = 0; i < BITS; ++i) bootsCOPY(&r[17 * BITS + i], &y[i], bk);
    for (int i = 0; i < BITS; ++i) bootsAND(&r[17 * BITS + i], &r[17 * BITS + i], &x[i], bk);

    f = open_or_die(in_dir(dir, "answer.data"), "wb");
    for (int i = 0; i < NRES * BITS; ++i) export_gate_bootstrapping_ciphertext_toFile(f, &r[i], params);
    fclose(f);
    delete_gate_bootstrapping_ciphertext_array(NRES * BITS, r);
    delete_gate_bootstrapping_ciphertext_array(BITS, y);
    delete_gate_bootstrapping_ciphertext_array(BITS, x);
    delete_gate_bootstrapping_cloud_keyset(bk);
    return 0;
}

static int verify(const char* dir, uint16_t x, uint16_t y) {
    FILE* f = open_or_die(in_dir(dir, "secret.key"), "rb");
    TFheGateBootstrappingSecretKeySet* key = new_tfheGateBootstrappingSecretKeySet_fromFile(f);
    fclose(f);
    if (!key) return 4;
    const TFheGateBootstrappingParameterSet* params = key->params;
    LweSample* r = new_gate_bootstrapping_ciphertext_array(NRES * BITS, params);
    f = open_or_die(in_dir(dir, "answer.data"), "rb");
    for (int i = 0; i < NRES * BITS; ++i) import_gate_bootstrapping_ciphertext_fromFile(f, &r[i], params);
    fclose(f);
    const uint16_t nx = (uint16_t)~x;
    const uint16_t want[NRES] = {
        (uint16_t)(x | y), (uint16_t)(x & y), (uint16_t)(x ^ y), (uint16_t)~(x & y),
        (uint16_t)~(x | y), (uint16_t)~(x ^ y), (uint16_t)(nx & y), (uint16_t)(x & (uint16_t)~y),
        (uint16_t)(nx | y), (uint16_t)(x | (uint16_t)~y), nx, y, 0x5A5A,
        (uint16_t)(x < y ? x : y), (uint16_t)(x + y), (uint16_t)(x ^ y),
        (uint16_t)((x & y) | nx), (uint16_t)(x & y)};
    int bad = 0;
    for (int k = 0; k < NRES; ++k) {
        uint16_t got = 0;
        for (int i = 0; i < BITS; ++i) got |= (uint16_t)(bootsSymDecrypt(&r[k * BITS + i], key) << i);
        printf("result %2d: %5u (want %5u)%s\n", k, got, want[k], got == want[k] ? "" : "  WRONG");
        bad += got != want[k];
    }
    delete_gate_bootstrapping_ciphertext_array(NRES * BITS, r);
    delete_gate_bootstrapping_secret_keyset(key);
    return bad ? 1 : 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s DIR client|cloud|verify|all [x y]\n", argv[0]);
        return 2;
    }
    const char* dir = argv[1];
    const uint16_t x = argc > 4 ? (uint16_t)atoi(argv[3]) : 499;
    const uint16_t y = argc > 4 ? (uint16_t)atoi(argv[4]) : 388;
    const char* what = argv[2];
    int rc = 0;
    if (!strcmp(what, "client") || !strcmp(what, "all")) rc = client(dir, x, y);
    if (!rc && (!strcmp(what, "cloud") || !strcmp(what, "all"))) rc = cloud(dir);
    if (!rc && (!strcmp(what, "verify") || !strcmp(what, "all"))) rc = verify(dir, x, y);
    return rc;
}
