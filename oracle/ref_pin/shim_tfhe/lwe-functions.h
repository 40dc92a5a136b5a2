// Stand-in for the upstream lwe-functions header: declarations matching the
// definitions in kernel/src/lwe-functions.cpp.
#ifndef REF_PIN_LWE_FUNCTIONS_H
#define REF_PIN_LWE_FUNCTIONS_H
#include "lwekey.h"
#include "lwesamples.h"
#include "numeric_functions.h"
EXPORT void lweKeyGen(LweKey* result);
EXPORT void lweSymEncrypt(LweSample* result, Torus32 message, double alpha, const LweKey* key);
EXPORT void lweSymEncryptWithExternalNoise(LweSample* result, Torus32 message, double noise,
                                           double alpha, const LweKey* key);
EXPORT Torus32 lwePhase(const LweSample* sample, const LweKey* key);
EXPORT Torus32 lweSymDecrypt(const LweSample* sample, const LweKey* key, const int32_t Msize);
EXPORT void lweClear(LweSample* result, const LweParams* params);
EXPORT void lweCopy(LweSample* result, const LweSample* sample, const LweParams* params);
EXPORT void lweNegate(LweSample* result, const LweSample* sample, const LweParams* params);
EXPORT void lweNoiselessTrivial(LweSample* result, Torus32 mu, const LweParams* params);
EXPORT void lweAddTo(LweSample* result, const LweSample* sample, const LweParams* params);
EXPORT void lweSubTo(LweSample* result, const LweSample* sample, const LweParams* params);
EXPORT void lweAddMulTo(LweSample* result, int32_t p, const LweSample* sample, const LweParams* params);
EXPORT void lweSubMulTo(LweSample* result, int32_t p, const LweSample* sample, const LweParams* params);
#endif
