/*
 * nova-gb300: Perseus over host buffers.
 *
 * Struct byte-identical to include/nova/pomdp/algorithms/pomdp_perseus_cpu.h:47-62.
 * The single-belief backup and the re-scoring of the remaining beliefs run
 * on the GB300; belief sampling uses the C library rand() exactly as the
 * reference does, so a caller that seeds srand() gets the same sequence.
 */
#ifndef NOVA_POMDP_PERSEUS_CPU_H
#define NOVA_POMDP_PERSEUS_CPU_H

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDPPerseusCPU {
    float *GammaInitial;

    unsigned int currentHorizon;

    unsigned int rGamma;
    unsigned int rGammaPrime;
    unsigned int rTilde;
    unsigned int *BTilde;

    float *Gamma;
    float *GammaPrime;
    unsigned int *pi;
    unsigned int *piPrime;
} POMDPPerseusCPU;

/* Replaces pomdp_perseus_initialize_cpu (pomdp_perseus_cpu.h:70, pomdp_perseus_cpu.cpp:183-219). */
NOVA_API int pomdp_perseus_initialize_cpu(const POMDP *pomdp, POMDPPerseusCPU *per);

/* Replaces pomdp_perseus_execute_cpu (pomdp_perseus_cpu.h:79, pomdp_perseus_cpu.cpp:222-270). */
NOVA_API int pomdp_perseus_execute_cpu(const POMDP *pomdp, POMDPPerseusCPU *per, POMDPAlphaVectors *policy);

/* Replaces pomdp_perseus_uninitialize_cpu (pomdp_perseus_cpu.h:88, pomdp_perseus_cpu.cpp:273-309). */
NOVA_API int pomdp_perseus_uninitialize_cpu(const POMDP *pomdp, POMDPPerseusCPU *per);

/* Replaces pomdp_perseus_update_cpu (pomdp_perseus_cpu.h:96, pomdp_perseus_cpu.cpp:312-429).
 * Returns NOVA_CONVERGED when the horizon step completes. */
NOVA_API int pomdp_perseus_update_cpu(const POMDP *pomdp, POMDPPerseusCPU *per);

/* Replaces pomdp_perseus_get_policy_cpu (pomdp_perseus_cpu.h:106, pomdp_perseus_cpu.cpp:432-461). */
NOVA_API int pomdp_perseus_get_policy_cpu(const POMDP *pomdp, POMDPPerseusCPU *per, POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
