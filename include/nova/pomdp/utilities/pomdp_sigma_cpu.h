/*
 * nova-gb300: sigma approximation of the belief set (computed on the GPU).
 */
#ifndef NOVA_POMDP_SIGMA_CPU_H
#define NOVA_POMDP_SIGMA_CPU_H

#include <nova/pomdp/pomdp.h>

NOVA_NS_BEGIN

/* Replaces pomdp_sigma_cpu (pomdp_sigma_cpu.h:43, pomdp_sigma_cpu.cpp:49-118):
 * every belief keeps its numDesiredNonZeroValues largest values, renormalised;
 * sigma = min(1, min over beliefs of the kept mass). Equal values keep their
 * support order (the reference's std::sort leaves their order unspecified);
 * beliefs with fewer entries than asked are padded with -1/0 (the reference
 * reads past its vector there). The C++ reference takes `float &sigma`. */
#ifdef __cplusplus
NOVA_API int pomdp_sigma_cpu(POMDP *pomdp, unsigned int numDesiredNonZeroValues, float &sigma);
#else
NOVA_API int pomdp_sigma_cpu(POMDP *pomdp, unsigned int numDesiredNonZeroValues, float *sigma);
#endif

NOVA_NS_END

#endif
