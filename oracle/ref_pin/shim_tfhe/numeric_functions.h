// Stand-in for the upstream numeric_functions header: declarations matching
// the definitions in kernel/src/numeric-functions.cpp.
#ifndef REF_PIN_NUMERIC_FUNCTIONS_H
#define REF_PIN_NUMERIC_FUNCTIONS_H
#include "tfhe_core.h"

const int64_t _two31 = INT64_C(1) << 31;
const int64_t _two32 = INT64_C(1) << 32;
const double _two31_double = (double)_two31;
const double _two32_double = (double)_two32;

extern std::default_random_engine generator;
extern std::uniform_int_distribution<Torus32> uniformTorus32_distrib;
extern std::uniform_int_distribution<int32_t> uniformInt_distrib;

EXPORT void tfhe_random_generator_setSeed(uint32_t* values, int32_t size);
EXPORT Torus32 gaussian32(Torus32 message, double sigma);
EXPORT Torus32 dtot32(double d);
EXPORT double t32tod(Torus32 x);
EXPORT Torus32 approxPhase(Torus32 phase, int32_t Msize);
EXPORT int32_t modSwitchFromTorus32(Torus32 phase, int32_t Msize);
EXPORT Torus32 modSwitchToTorus32(int32_t mu, int32_t Msize);
#endif
