/*
 * nova-gb300: MDP value iteration over host buffers.
 *
 * Struct byte-identical to include/nova/mdp/algorithms/mdp_vi_cpu.h:42-50.
 * The Bellman sweep runs on the GB300; after every call V, VPrime and pi are
 * valid host arrays, as the reference's tests read them directly.
 */
#ifndef NOVA_MDP_VI_CPU_H
#define NOVA_MDP_VI_CPU_H

#include <nova/mdp/mdp.h>
#include <nova/mdp/policies/mdp_value_function.h>

NOVA_NS_BEGIN

typedef struct NovaMDPVICPU {
    float *VInitial;

    unsigned int currentHorizon;

    float *V;
    float *VPrime;
    unsigned int *pi;
} MDPVICPU;

/* Replaces mdp_vi_initialize_cpu (mdp_vi_cpu.h:58, mdp_vi_cpu.cpp:66-98). */
NOVA_API int mdp_vi_initialize_cpu(const MDP *mdp, MDPVICPU *vi);

/* Replaces mdp_vi_execute_cpu (mdp_vi_cpu.h:67, mdp_vi_cpu.cpp:101-152). */
NOVA_API int mdp_vi_execute_cpu(const MDP *mdp, MDPVICPU *vi, MDPValueFunction *policy);

/* Replaces mdp_vi_uninitialize_cpu (mdp_vi_cpu.h:75, mdp_vi_cpu.cpp:155-182). */
NOVA_API int mdp_vi_uninitialize_cpu(const MDP *mdp, MDPVICPU *vi);

/* Replaces mdp_vi_update_cpu (mdp_vi_cpu.h:83, mdp_vi_cpu.cpp:185-196). */
NOVA_API int mdp_vi_update_cpu(const MDP *mdp, MDPVICPU *vi);

/* Replaces mdp_vi_get_policy_cpu (mdp_vi_cpu.h:93, mdp_vi_cpu.cpp:199-223). */
NOVA_API int mdp_vi_get_policy_cpu(const MDP *mdp, MDPVICPU *vi, MDPValueFunction *policy);

NOVA_NS_END

#endif
