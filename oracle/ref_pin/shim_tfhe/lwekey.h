// Stand-in for the upstream LweKey (fields used by the reference).
#ifndef REF_PIN_LWEKEY_H
#define REF_PIN_LWEKEY_H
#include "lweparams.h"
struct LweKey {
    const LweParams* params;
    int32_t* key;
    explicit LweKey(const LweParams* p) : params(p), key(new int32_t[p->n]) {}
    ~LweKey() { delete[] key; }
    LweKey(const LweKey&) = delete;
    LweKey& operator=(const LweKey&) = delete;
};
#endif
