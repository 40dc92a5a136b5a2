// Stand-in for the upstream LweParams (fields used by the reference).
#ifndef REF_PIN_LWEPARAMS_H
#define REF_PIN_LWEPARAMS_H
#include "tfhe_core.h"
struct LweParams {
    const int32_t n;
    const double alpha_min;
    const double alpha_max;
    LweParams(int32_t n_, double min_, double max_) : n(n_), alpha_min(min_), alpha_max(max_) {}
};
#endif
