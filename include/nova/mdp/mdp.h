/*
 * nova-gb300: the MDP model container.
 *
 * Byte-identical to the reference struct (include/nova/mdp/mdp.h:53-75).
 *   S, T : [n][m][ns]  successor state / probability; a row (s,a) ends at its
 *                      first negative successor.
 *   R    : [n][m]      reward R(s, a).
 */
#ifndef NOVA_MDP_H
#define NOVA_MDP_H

#include <nova/nova_abi.h>

NOVA_NS_BEGIN

typedef struct NovaMDP {
    unsigned int n;
    unsigned int ns;
    unsigned int m;

    float gamma;
    unsigned int horizon;
    float epsilon;

    unsigned int s0;
    unsigned int ng;
    unsigned int *goals;

    int *S;
    float *T;
    float *R;

    unsigned int *d_goals;

    int *d_S;
    float *d_T;
    float *d_R;
} MDP;

NOVA_NS_END

#endif
