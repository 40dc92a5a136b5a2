// ref_driver_tfhe.cpp -- flat-array entry points over the reference's own CPU
// functions (kernel/src/numeric-functions.cpp, lwe-functions.cpp,
// lwe-keyswitch-functions.cpp), compiled unmodified against the stand-in
// headers in shim_tfhe/.  Test infrastructure: the oracle pin tests call
// these to check the oracle's restatement against the reference code.
#include <string.h>

#include "lwe-functions.h"
#include "lwekeyswitch.h"
#include "numeric_functions.h"

extern "C" {

void refu_lwe_keygen(int32_t n, int32_t* out) {
    LweParams p(n, 0., 0.);
    LweKey k(&p);
    lweKeyGen(&k);
    memcpy(out, k.key, sizeof(int32_t) * n);
}

void refu_lwe_encrypt(int32_t n, const int32_t* key, int32_t message, double alpha, int32_t* out) {
    LweParams p(n, alpha, 0.);
    LweKey k(&p);
    memcpy(k.key, key, sizeof(int32_t) * n);
    LweSample s(&p);
    lweSymEncrypt(&s, message, alpha, &k);
    memcpy(out, s.a, sizeof(int32_t) * n);
    out[n] = s.b;
}

int32_t refu_lwe_phase(int32_t n, const int32_t* key, const int32_t* sample) {
    LweParams p(n, 0., 0.);
    LweKey k(&p);
    memcpy(k.key, key, sizeof(int32_t) * n);
    LweSample s(&p);
    memcpy(s.a, sample, sizeof(int32_t) * n);
    s.b = sample[n];
    return lwePhase(&s, &k);
}

// lweCreateKeySwitchKey from in_key (n_in bits) to out_key (n_out), noise
// alpha; out: [n_in][t][base][n_out + 1].
void refu_create_ks_key(int32_t n_in, const int32_t* in_key, int32_t n_out, const int32_t* out_key,
                        int32_t t, int32_t basebit, double alpha, int32_t* out) {
    LweParams pin(n_in, 0., 0.), pout(n_out, alpha, 0.);
    LweKey kin(&pin), kout(&pout);
    memcpy(kin.key, in_key, sizeof(int32_t) * n_in);
    memcpy(kout.key, out_key, sizeof(int32_t) * n_out);
    LweKeySwitchKey* ks = (LweKeySwitchKey*)malloc(sizeof(LweKeySwitchKey));
    init_LweKeySwitchKey(ks, n_in, t, basebit, &pout);
    lweCreateKeySwitchKey(ks, &kin, &kout);
    const int32_t rows = n_in * t * (1 << basebit);
    for (int32_t r = 0; r < rows; ++r) {
        memcpy(out + (size_t)r * (n_out + 1), ks->ks0_raw[r].a, sizeof(int32_t) * n_out);
        out[(size_t)r * (n_out + 1) + n_out] = ks->ks0_raw[r].b;
    }
    destroy_LweKeySwitchKey(ks);
    free(ks);
}

// lweKeySwitch with a table in the flat layout above.
void refu_keyswitch(int32_t n_in, int32_t n_out, int32_t t, int32_t basebit, const int32_t* table,
                    const int32_t* in, int32_t* out) {
    LweParams pin(n_in, 0., 0.), pout(n_out, 0., 0.);
    LweKeySwitchKey* ks = (LweKeySwitchKey*)malloc(sizeof(LweKeySwitchKey));
    init_LweKeySwitchKey(ks, n_in, t, basebit, &pout);
    const int32_t rows = n_in * t * (1 << basebit);
    for (int32_t r = 0; r < rows; ++r) {
        memcpy(ks->ks0_raw[r].a, table + (size_t)r * (n_out + 1), sizeof(int32_t) * n_out);
        ks->ks0_raw[r].b = table[(size_t)r * (n_out + 1) + n_out];
    }
    LweSample x(&pin), res(&pout);
    memcpy(x.a, in, sizeof(int32_t) * n_in);
    x.b = in[n_in];
    lweKeySwitch(&res, ks, &x);
    memcpy(out, res.a, sizeof(int32_t) * n_out);
    out[n_out] = res.b;
    destroy_LweKeySwitchKey(ks);
    free(ks);
}

// The testbench's OR combination (tfhe_blindRotate_FFT_tb.cpp:271-276):
// (0, c) + ca + cb with lweNoiselessTrivial and lweAddTo.
void refu_or_combination(int32_t n, int32_t c, const int32_t* ca, const int32_t* cb, int32_t* out) {
    LweParams p(n, 0., 0.);
    LweSample r(&p), a(&p), b(&p);
    memcpy(a.a, ca, sizeof(int32_t) * n);
    a.b = ca[n];
    memcpy(b.a, cb, sizeof(int32_t) * n);
    b.b = cb[n];
    lweNoiselessTrivial(&r, c, &p);
    lweAddTo(&r, &a, &p);
    lweAddTo(&r, &b, &p);
    memcpy(out, r.a, sizeof(int32_t) * n);
    out[n] = r.b;
}

}  // extern "C"
