// Stand-in for the upstream LweKeySwitchKey: a flat array of n*t*base
// samples (ks0_raw) with ks[i][j][h] = ks0_raw + (i t + j) base + h, the
// addressing the reference's key switch uses.
#ifndef REF_PIN_LWEKEYSWITCH_H
#define REF_PIN_LWEKEYSWITCH_H
#include "lwekey.h"
#include "lwesamples.h"
struct LweKeySwitchKey {
    int32_t n, t, basebit, base;
    const LweParams* out_params;
    LweSample* ks0_raw;
    LweSample** ks1_raw;
    LweSample*** ks;
    LweKeySwitchKey(int32_t n_, int32_t t_, int32_t basebit_, const LweParams* out, LweSample* raw)
        : n(n_), t(t_), basebit(basebit_), base(1 << basebit_), out_params(out), ks0_raw(raw) {
        ks1_raw = new LweSample*[(size_t)n * t];
        ks = new LweSample**[n];
        for (int32_t p = 0; p < n * t; ++p) ks1_raw[p] = ks0_raw + (size_t)base * p;
        for (int32_t p = 0; p < n; ++p) ks[p] = ks1_raw + (size_t)t * p;
    }
    ~LweKeySwitchKey() {
        delete[] ks1_raw;
        delete[] ks;
    }
};
EXPORT void init_LweKeySwitchKey(LweKeySwitchKey* obj, int32_t n, int32_t t, int32_t basebit,
                                 const LweParams* out_params);
EXPORT void destroy_LweKeySwitchKey(LweKeySwitchKey* obj);
EXPORT void lweCreateKeySwitchKey(LweKeySwitchKey* result, const LweKey* in_key, const LweKey* out_key);
EXPORT void lweKeySwitch(LweSample* result, const LweKeySwitchKey* ks, const LweSample* sample);
#endif
