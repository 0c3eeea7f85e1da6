/*
 * nova-gb300: PBVI over host buffers.
 *
 * Struct byte-identical to include/nova/pomdp/algorithms/pomdp_pbvi_cpu.h:42-50.
 * In this library the backup itself runs on the GB300 (the same kernels as
 * the _gpu entry points); these entry points keep the reference's host-buffer
 * contract: the model arrays are the host arrays of the POMDP, and after
 * every call Gamma, GammaPrime and pi are valid host arrays.
 */
#ifndef NOVA_POMDP_PBVI_CPU_H
#define NOVA_POMDP_PBVI_CPU_H

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDPPBVICPU {
    float *GammaInitial;

    unsigned int currentHorizon;

    float *Gamma;
    float *GammaPrime;
    unsigned int *pi;
} POMDPPBVICPU;

/* Replaces pomdp_pbvi_initialize_cpu (pomdp_pbvi_cpu.h:58, pomdp_pbvi_cpu.cpp:165-183). */
NOVA_API int pomdp_pbvi_initialize_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi);

/* Replaces pomdp_pbvi_execute_cpu (pomdp_pbvi_cpu.h:67, pomdp_pbvi_cpu.cpp:186-229). */
NOVA_API int pomdp_pbvi_execute_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi, POMDPAlphaVectors *policy);

/* Replaces pomdp_pbvi_uninitialize_cpu (pomdp_pbvi_cpu.h:75, pomdp_pbvi_cpu.cpp:232-254). */
NOVA_API int pomdp_pbvi_uninitialize_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi);

/* Replaces pomdp_pbvi_update_cpu (pomdp_pbvi_cpu.h:83, pomdp_pbvi_cpu.cpp:257-273). */
NOVA_API int pomdp_pbvi_update_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi);

/* Replaces pomdp_pbvi_get_policy_cpu (pomdp_pbvi_cpu.h:93, pomdp_pbvi_cpu.cpp:276-300). */
NOVA_API int pomdp_pbvi_get_policy_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi, POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
