// Stand-in for the upstream macro that generates new_/delete_ helpers from a
// type's init_/destroy_ functions (used by kernel/src/lwe-functions.cpp:279-281).
#ifndef REF_PIN_TFHE_GENERIC_TEMPLATES_H
#define REF_PIN_TFHE_GENERIC_TEMPLATES_H
#include <stdlib.h>
#define USE_DEFAULT_CONSTRUCTOR_DESTRUCTOR_IMPLEMENTATIONS1(TYPE, PARAM1)                       \
    EXPORT TYPE* new_##TYPE(const PARAM1* p1) {                                               \
        TYPE* o = (TYPE*)malloc(sizeof(TYPE));                                                \
        init_##TYPE(o, p1);                                                                   \
        return o;                                                                             \
    }                                                                                         \
    EXPORT TYPE* new_##TYPE##_array(int32_t nb, const PARAM1* p1) {                           \
        TYPE* o = (TYPE*)malloc((size_t)nb * sizeof(TYPE));                                   \
        for (int32_t i = 0; i < nb; ++i) init_##TYPE(o + i, p1);                              \
        return o;                                                                             \
    }                                                                                         \
    EXPORT void delete_##TYPE(TYPE* o) {                                                      \
        destroy_##TYPE(o);                                                                    \
        free(o);                                                                              \
    }                                                                                         \
    EXPORT void delete_##TYPE##_array(int32_t nb, TYPE* o) {                                  \
        for (int32_t i = 0; i < nb; ++i) destroy_##TYPE(o + i);                               \
        free(o);                                                                              \
    }
#endif
