// Stand-in for the upstream TFHE core header (test infrastructure): the
// Torus32 type and the EXPORT macro the reference's CPU files use.  EXPORT
// gives C linkage so the pin driver (and ctypes) can call the functions.
#ifndef REF_PIN_TFHE_CORE_H
#define REF_PIN_TFHE_CORE_H
#include <stdint.h>
#include <stdlib.h>

#include <random>

typedef int32_t Torus32;
#define EXPORT extern "C"

struct LweParams;
struct LweKey;
struct LweSample;
struct LweKeySwitchKey;
#endif
