/*
 * nova-gb300: MDP value function (the get_policy target of value iteration).
 *
 * Struct byte-identical to include/nova/mdp/policies/mdp_value_function.h:48-57.
 * r == 0 means dense V and pi of length n and S == nullptr.
 */
#ifndef NOVA_MDP_VALUE_FUNCTION_H
#define NOVA_MDP_VALUE_FUNCTION_H

#include <nova/nova_abi.h>

NOVA_NS_BEGIN

typedef struct NovaMDPValueFunction {
    unsigned int n;
    unsigned int m;
    unsigned int r;

    unsigned int *S;
    float *V;
    unsigned int *pi;
} MDPValueFunction;

/* Replaces mdp_value_function_initialize (mdp_value_function.h:65-66,
 * mdp_value_function.cpp:34-57). */
NOVA_API int mdp_value_function_initialize(MDPValueFunction *policy,
        unsigned int n, unsigned int m, unsigned int r);

/* Replaces mdp_value_function_uninitialize (mdp_value_function.h:72,
 * mdp_value_function.cpp:60-87). */
NOVA_API int mdp_value_function_uninitialize(MDPValueFunction *policy);

NOVA_NS_END

#endif
