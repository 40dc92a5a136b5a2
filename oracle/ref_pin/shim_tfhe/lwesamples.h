// Stand-in for the upstream LweSample (fields used by the reference) and the
// allocation helpers the key switch uses.
#ifndef REF_PIN_LWESAMPLES_H
#define REF_PIN_LWESAMPLES_H
#include "lweparams.h"
struct LweSample {
    Torus32* a;
    Torus32 b;
    double current_variance;
    explicit LweSample(const LweParams* p) : a(new Torus32[p->n]), b(0), current_variance(0.) {}
    ~LweSample() { delete[] a; }
    LweSample(const LweSample&) = delete;
    LweSample& operator=(const LweSample&) = delete;
};
EXPORT void init_LweSample(LweSample* obj, const LweParams* params);
EXPORT void destroy_LweSample(LweSample* obj);
EXPORT LweSample* new_LweSample(const LweParams* params);
EXPORT void delete_LweSample(LweSample* obj);
EXPORT LweSample* new_LweSample_array(int32_t nbelts, const LweParams* params);
EXPORT void delete_LweSample_array(int32_t nbelts, LweSample* obj);
EXPORT void init_LweKey(LweKey* obj, const LweParams* params);
EXPORT void destroy_LweKey(LweKey* obj);
#endif
