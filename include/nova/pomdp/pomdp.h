/*
 * nova-gb300: the POMDP model container.
 *
 * Byte-identical to the reference struct (include/nova/pomdp/pomdp.h:61-85).
 * Layouts of the arrays (all row-major, 32-bit):
 *   S, T : [n][m][ns]  successor state / probability; a row (s,a) ends at its
 *                      first negative successor.
 *   O    : [m][n][z]   observation probability O(a, s', o).
 *   R    : [n][m]      reward R(s, a).
 *   Z, B : [r][rz]     belief support state / probability; a row ends at its
 *                      first negative state.
 * The d_* fields hold device copies made by pomdp_initialize_gpu.
 */
#ifndef NOVA_POMDP_H
#define NOVA_POMDP_H

#include <nova/nova_abi.h>

NOVA_NS_BEGIN

typedef struct NovaPOMDP {
    unsigned int n;
    unsigned int ns;
    unsigned int m;
    unsigned int z;
    unsigned int r;
    unsigned int rz;

    float gamma;
    unsigned int horizon;

    int *S;
    float *T;
    float *O;
    float *R;
    int *Z;
    float *B;

    int *d_S;
    float *d_T;
    float *d_O;
    float *d_R;
    int *d_Z;
    float *d_B;
} POMDP;

NOVA_NS_END

#endif
