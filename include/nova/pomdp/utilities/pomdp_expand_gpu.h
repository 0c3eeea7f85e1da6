/*
 * nova-gb300: random belief expansion from belief 0 (the reference's GPU-named form).
 */
#ifndef NOVA_POMDP_EXPAND_GPU_H
#define NOVA_POMDP_EXPAND_GPU_H

#include <nova/pomdp/pomdp.h>

NOVA_NS_BEGIN

/* Replaces pomdp_expand_random_gpu (pomdp_expand_gpu.h:47-48, pomdp_expand_gpu.cu:127-215):
 * Bnew (allocated with new[], [numDesiredBeliefPoints][n]) holds belief 0 and
 * then beliefs of random trajectories that start at belief 0;
 * maxNonZeroValues is the largest support among the expanded ones. numThreads
 * is accepted for the ABI (launch shapes are fixed). The C++ reference takes
 * `unsigned int &` and `float *&`, i.e. pointers at the C ABI. */
#ifdef __cplusplus
NOVA_API int pomdp_expand_random_gpu(const POMDP *pomdp, unsigned int numThreads,
        unsigned int numDesiredBeliefPoints, unsigned int &maxNonZeroValues, float *&Bnew);
#else
NOVA_API int pomdp_expand_random_gpu(const POMDP *pomdp, unsigned int numThreads,
        unsigned int numDesiredBeliefPoints, unsigned int *maxNonZeroValues, float **Bnew);
#endif

NOVA_NS_END

#endif
