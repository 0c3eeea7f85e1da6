/*
 * nova-gb300: alpha-vector policy (the get_policy target of PBVI / Perseus).
 *
 * Struct byte-identical to include/nova/pomdp/policies/pomdp_alpha_vectors.h:39-47.
 * Gamma is [r][n], pi is [r]; both are host arrays owned by the policy.
 */
#ifndef NOVA_POMDP_ALPHA_VECTORS_H
#define NOVA_POMDP_ALPHA_VECTORS_H

#include <nova/nova_abi.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDPAlphaVectors {
    unsigned int n;
    unsigned int m;
    unsigned int r;

    float *Gamma;
    unsigned int *pi;
} POMDPAlphaVectors;

/* Replaces pomdp_alpha_vectors_initialize (pomdp_alpha_vectors.h:55-56,
 * pomdp_alpha_vectors.cpp:34-49): fails unless Gamma and pi are null. */
NOVA_API int pomdp_alpha_vectors_initialize(POMDPAlphaVectors *policy,
        unsigned int n, unsigned int m, unsigned int r);

/* Replaces pomdp_alpha_vectors_value_and_action (pomdp_alpha_vectors.h:65-66,
 * pomdp_alpha_vectors.cpp:52-79): V(b) = max_i Gamma_i . b over a host
 * policy, strict '>' so the lowest index wins ties. The C++ reference passes
 * Vb and a by reference, which is a pointer at the C ABI. */
#ifdef __cplusplus
NOVA_API int pomdp_alpha_vectors_value_and_action(const POMDPAlphaVectors *policy,
        const float *b, float &Vb, unsigned int &a);
#else
NOVA_API int pomdp_alpha_vectors_value_and_action(const POMDPAlphaVectors *policy,
        const float *b, float *Vb, unsigned int *a);
#endif

/* Replaces pomdp_alpha_vectors_uninitialize (pomdp_alpha_vectors.h:72,
 * pomdp_alpha_vectors.cpp:82-107). */
NOVA_API int pomdp_alpha_vectors_uninitialize(POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
