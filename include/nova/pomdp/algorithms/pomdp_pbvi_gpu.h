/*
 * nova-gb300: PBVI over device buffers (the GB300 hot path).
 *
 * Struct byte-identical to include/nova/pomdp/algorithms/pomdp_pbvi_gpu.h:44-55.
 * numThreads is validated (multiple of 32) for compatibility; tile shapes
 * come from the library, not from it. d_alphaBA is not used and stays null:
 * the library keeps its own per-solver workspace.
 */
#ifndef NOVA_POMDP_PBVI_GPU_H
#define NOVA_POMDP_PBVI_GPU_H

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDPPBVIGPU {
    float *GammaInitial;
    unsigned int numThreads;

    unsigned int currentHorizon;

    float *d_Gamma;
    float *d_GammaPrime;
    unsigned int *d_pi;
    float *d_alphaBA;
} POMDPPBVIGPU;

/* Replaces pomdp_pbvi_initialize_gpu (pomdp_pbvi_gpu.h:63, pomdp_pbvi_gpu.cu:213-257).
 * Idempotent: a second call on the same struct releases what the first made. */
NOVA_API int pomdp_pbvi_initialize_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi);

/* Replaces pomdp_pbvi_execute_gpu (pomdp_pbvi_gpu.h:72, pomdp_pbvi_gpu.cu:260-309). */
NOVA_API int pomdp_pbvi_execute_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, POMDPAlphaVectors *policy);

/* Replaces pomdp_pbvi_uninitialize_gpu (pomdp_pbvi_gpu.h:81, pomdp_pbvi_gpu.cu:312-358). */
NOVA_API int pomdp_pbvi_uninitialize_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi);

/* Replaces pomdp_pbvi_update_gpu (pomdp_pbvi_gpu.h:89, pomdp_pbvi_gpu.cu:361-441). */
NOVA_API int pomdp_pbvi_update_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi);

/* Replaces pomdp_pbvi_get_policy_gpu (pomdp_pbvi_gpu.h:99, pomdp_pbvi_gpu.cu:444-484). */
NOVA_API int pomdp_pbvi_get_policy_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
