/*
 * nova-gb300: MDP value iteration over device buffers (the GB300 hot path).
 *
 * Struct byte-identical to include/nova/mdp/algorithms/mdp_vi_gpu.h:43-52.
 * numThreads is validated (multiple of 32) for compatibility only.
 */
#ifndef NOVA_MDP_VI_GPU_H
#define NOVA_MDP_VI_GPU_H

#include <nova/mdp/mdp.h>
#include <nova/mdp/policies/mdp_value_function.h>

NOVA_NS_BEGIN

typedef struct NovaMDPVIGPU {
    float *VInitial;
    unsigned int numThreads;

    unsigned int currentHorizon;

    float *d_V;
    float *d_VPrime;
    unsigned int *d_pi;
} MDPVIGPU;

/* Replaces mdp_vi_initialize_gpu (mdp_vi_gpu.h:60, mdp_vi_gpu.cu:90-160). */
NOVA_API int mdp_vi_initialize_gpu(const MDP *mdp, MDPVIGPU *vi);

/* Replaces mdp_vi_execute_gpu (mdp_vi_gpu.h:69, mdp_vi_gpu.cu:163-221). */
NOVA_API int mdp_vi_execute_gpu(const MDP *mdp, MDPVIGPU *vi, MDPValueFunction *policy);

/* Replaces mdp_vi_uninitialize_gpu (mdp_vi_gpu.h:77, mdp_vi_gpu.cu:224-266). */
NOVA_API int mdp_vi_uninitialize_gpu(const MDP *mdp, MDPVIGPU *vi);

/* Replaces mdp_vi_update_gpu (mdp_vi_gpu.h:85, mdp_vi_gpu.cu:269-307). */
NOVA_API int mdp_vi_update_gpu(const MDP *mdp, MDPVIGPU *vi);

/* Replaces mdp_vi_get_policy_gpu (mdp_vi_gpu.h:95, mdp_vi_gpu.cu:310-346). */
NOVA_API int mdp_vi_get_policy_gpu(const MDP *mdp, MDPVIGPU *vi, MDPValueFunction *policy);

NOVA_NS_END

#endif
