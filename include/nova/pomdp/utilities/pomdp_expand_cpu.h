/*
 * nova-gb300: belief-set expansion (host-array POMDPs; computed on the GPU).
 */
#ifndef NOVA_POMDP_EXPAND_CPU_H
#define NOVA_POMDP_EXPAND_CPU_H

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

/* Replaces pomdp_expand_random_cpu (pomdp_expand_cpu.h:43, pomdp_expand_cpu.cpp:81-150):
 * numBeliefsToAdd beliefs from random trajectories (libc rand(), seeded with
 * time(nullptr) as in the reference unless nova_gb300_expand_seed fixed a
 * seed), appended to Z/B. */
NOVA_API int pomdp_expand_random_cpu(POMDP *pomdp, unsigned int numBeliefsToAdd);

/* Replaces pomdp_expand_distinct_beliefs_cpu (pomdp_expand_cpu.h:52,
 * pomdp_expand_cpu.cpp:153-241): for every belief, the successor b'(b, a, o)
 * farthest in L1 from the set; r beliefs appended. A belief with no valid
 * (a, o) adds a zero row (the reference copies an uninitialised buffer). */
NOVA_API int pomdp_expand_distinct_beliefs_cpu(POMDP *pomdp);

/* Replaces pomdp_expand_pema_cpu (pomdp_expand_cpu.h:61, pomdp_expand_cpu.cpp:244-383):
 * one belief chosen by PEMA's error bound under the given policy, appended. */
NOVA_API int pomdp_expand_pema_cpu(POMDP *pomdp, const POMDPAlphaVectors *policy);

NOVA_NS_END

#endif
