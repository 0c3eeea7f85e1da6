/*
 * nova-gb300: host-side POMDP model allocation.
 */
#ifndef NOVA_POMDP_MODEL_CPU_H
#define NOVA_POMDP_MODEL_CPU_H

#include <nova/pomdp/pomdp.h>

NOVA_NS_BEGIN

/* Replaces pomdp_initialize_cpu (pomdp_model_cpu.h:47, pomdp_model_cpu.cpp:34-86):
 * allocates S,T,O,R,Z,B with new[]; S=-1, everything else 0. */
NOVA_API int pomdp_initialize_cpu(POMDP *pomdp, unsigned int n, unsigned int ns, unsigned int m,
        unsigned int z, unsigned int r, unsigned int rz, float gamma, unsigned int horizon);

/* Replaces pomdp_belief_update_cpu (pomdp_model_cpu.h:59, pomdp_model_cpu.cpp:89-137):
 * b' = normalise(O(a,.,o) * T(.,a,.)^T b); bp must be null on entry and is
 * allocated with new[]. The C++ reference takes `float *&bp`, i.e. a
 * `float **` at the C ABI. */
#ifdef __cplusplus
NOVA_API int pomdp_belief_update_cpu(const POMDP *pomdp, const float *b,
        unsigned int a, unsigned int o, float *&bp);
#else
NOVA_API int pomdp_belief_update_cpu(const POMDP *pomdp, const float *b,
        unsigned int a, unsigned int o, float **bp);
#endif

/* Replaces pomdp_add_new_raw_beliefs_cpu (pomdp_model_cpu.h:69, pomdp_model_cpu.cpp:157-227):
 * appends dense beliefs Bnew [numBeliefsToAdd][n] to Z/B, widening rz if needed. */
NOVA_API int pomdp_add_new_raw_beliefs_cpu(POMDP *pomdp, unsigned int numBeliefsToAdd, float *Bnew);

/* Replaces pomdp_uninitialize_cpu (pomdp_model_cpu.h:77, pomdp_model_cpu.cpp:230-277). */
NOVA_API int pomdp_uninitialize_cpu(POMDP *pomdp);

NOVA_NS_END

#endif
