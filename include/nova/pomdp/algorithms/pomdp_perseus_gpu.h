/*
 * nova-gb300: Perseus over device buffers.
 *
 * The reference has no GPU Perseus; this struct follows the reference's
 * POMDPPerseusCPU (include/nova/pomdp/algorithms/pomdp_perseus_cpu.h:47-62)
 * with device arrays, plus numThreads as in POMDPPBVIGPU. BTilde stays a
 * host array: beliefs are drawn on the host with the C library rand(), as in
 * pomdp_perseus_cpu.cpp:340-341, so a seeded srand() reproduces the
 * reference's sequence. Each update backs up one belief on the GB300 and
 * re-scores every belief there.
 */
#ifndef NOVA_POMDP_PERSEUS_GPU_H
#define NOVA_POMDP_PERSEUS_GPU_H

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDPPerseusGPU {
    float *GammaInitial;
    unsigned int numThreads;

    unsigned int currentHorizon;

    unsigned int rGamma;
    unsigned int rGammaPrime;
    unsigned int rTilde;
    unsigned int *BTilde;

    float *d_Gamma;
    float *d_GammaPrime;
    unsigned int *d_pi;
    unsigned int *d_piPrime;
} POMDPPerseusGPU;

/* New; mirrors pomdp_perseus_initialize_cpu (pomdp_perseus_cpu.cpp:183-219). */
NOVA_API int pomdp_perseus_initialize_gpu(const POMDP *pomdp, POMDPPerseusGPU *per);

/* New; mirrors pomdp_perseus_execute_cpu (pomdp_perseus_cpu.cpp:222-270). */
NOVA_API int pomdp_perseus_execute_gpu(const POMDP *pomdp, POMDPPerseusGPU *per, POMDPAlphaVectors *policy);

/* New; mirrors pomdp_perseus_uninitialize_cpu (pomdp_perseus_cpu.cpp:273-309). */
NOVA_API int pomdp_perseus_uninitialize_gpu(const POMDP *pomdp, POMDPPerseusGPU *per);

/* New; mirrors pomdp_perseus_update_cpu (pomdp_perseus_cpu.cpp:312-429).
 * Returns NOVA_CONVERGED when the horizon step completes. */
NOVA_API int pomdp_perseus_update_gpu(const POMDP *pomdp, POMDPPerseusGPU *per);

/* New; mirrors pomdp_perseus_get_policy_cpu (pomdp_perseus_cpu.cpp:432-461). */
NOVA_API int pomdp_perseus_get_policy_gpu(const POMDP *pomdp, POMDPPerseusGPU *per, POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
