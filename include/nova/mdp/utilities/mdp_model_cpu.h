/*
 * nova-gb300: host-side MDP model allocation.
 */
#ifndef NOVA_MDP_MODEL_CPU_H
#define NOVA_MDP_MODEL_CPU_H

#include <nova/mdp/mdp.h>

NOVA_NS_BEGIN

/* Replaces mdp_initialize_cpu (mdp_model_cpu.h:46, mdp_model_cpu.cpp:35-82). */
NOVA_API int mdp_initialize_cpu(MDP *mdp, unsigned int n, unsigned int ns, unsigned int m, float gamma,
        unsigned int horizon, float epsilon, unsigned int s0, unsigned int ng);

/* Replaces mdp_uninitialize_cpu (mdp_model_cpu.h:54, mdp_model_cpu.cpp:85-122). */
NOVA_API int mdp_uninitialize_cpu(MDP *mdp);

NOVA_NS_END

#endif
