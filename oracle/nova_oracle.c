/*
 * nova-gb300 ORACLE -- test infrastructure only.
 *
 * A plain-C restatement of kylewray/nova's CPU algorithms for the hot path,
 * used as the parity checker by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py. Nothing in the product library links or calls it.
 *
 * Parity is pinned: tests/test_oracle.py checks every function here bit for
 * bit against fixtures produced by the reference itself (its CPU sources
 * compiled by oracle/Makefile into oracle/_ref, run by
 * tests/golden/make_golden.py) and against the reference's unit-test values.
 *
 * Arithmetic is IEEE FP32 with every product and sum rounded separately
 * (build with -ffp-contract=off): the reference is built by g++ for x86-64
 * without FMA, and these functions reproduce its operation order exactly.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>
#include <unistd.h>

#define ORACLE_FLT_MIN (-1e+10f)   /* nova's FLT_MIN, include/nova/constants.h:34 */

/* ------------------------------------------------------------------------ */
/* PBVI, the reference's own loop structure                                  */
/* ------------------------------------------------------------------------ */

/* Follows pomdp_pbvi_update_compute_best_alpha_cpu, pomdp_pbvi_cpu.cpp:37-103.
 * bestj persists across observations (it is declared outside the o loop) and
 * is never assigned when no alpha beats the -1e10 sentinel; here it starts
 * at 0 in every call (the product library does the same). */
static void pbvi_best_alpha(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned rG, unsigned rz, float gamma,
                            const int *S, const float *T, const float *O, const int *Z, const float *B,
                            const float *Gamma, unsigned i, unsigned a, float *alpha, unsigned *bestjState,
                            unsigned *jstarOut) {
    unsigned bestj = 0;
    (void)bestjState;
    for (unsigned o = 0; o < z; o++) {
        float bestValue = ORACLE_FLT_MIN;
        for (unsigned j = 0; j < rG; j++) {
            float value = 0.0f;
            for (unsigned k = 0; k < rz; k++) {
                int s = Z[i * rz + k];
                if (s < 0) break;
                float Vtk = 0.0f;
                for (unsigned l = 0; l < ns; l++) {
                    int sp = S[s * m * ns + a * ns + l];
                    if (sp < 0) break;
                    float ot = O[a * n * z + sp * z + o] * T[s * m * ns + a * ns + l];
                    float p = ot * Gamma[j * n + sp];
                    Vtk = Vtk + p;
                }
                Vtk = Vtk * gamma;
                float q = Vtk * B[i * rz + k];
                value = value + q;
            }
            if (value > bestValue) {
                bestj = j;
                bestValue = value;
            }
        }
        if (jstarOut) jstarOut[o] = bestj;
        for (unsigned s = 0; s < n; s++) {
            float Vtk = 0.0f;
            for (unsigned l = 0; l < ns; l++) {
                int sp = S[s * m * ns + a * ns + l];
                if (sp < 0) break;
                float ot = O[a * n * z + sp * z + o] * T[s * m * ns + a * ns + l];
                float p = ot * Gamma[bestj * n + sp];
                Vtk = Vtk + p;
            }
            Vtk = Vtk * gamma;
            alpha[s] = alpha[s] + Vtk;
        }
    }
}

/* Follows pomdp_pbvi_update_step_cpu, pomdp_pbvi_cpu.cpp:106-162: one backup
 * of beliefs [i0, i1) against Gamma (r rows), writing GammaPrime rows and
 * pi. Rows/actions of beliefs that no action improves are left untouched. */
void oracle_pbvi_update_range(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                              const int *S, const float *T, const float *O, const float *R, const int *Z,
                              const float *B, const float *Gamma, float *GammaPrime, unsigned *pi, unsigned i0,
                              unsigned i1) {
    float *alpha = (float *)malloc(sizeof(float) * n);
    unsigned bestjState = 0;
    for (unsigned i = i0; i < i1; i++) {
        float bestValue = ORACLE_FLT_MIN;
        for (unsigned a = 0; a < m; a++) {
            for (unsigned s = 0; s < n; s++) alpha[s] = R[s * m + a];
            pbvi_best_alpha(n, ns, m, z, r, rz, gamma, S, T, O, Z, B, Gamma, i, a, alpha, &bestjState, NULL);
            float value = 0.0f;
            for (unsigned k = 0; k < rz; k++) {
                int s = Z[i * rz + k];
                if (s < 0) break;
                float q = alpha[s] * B[i * rz + k];
                value = value + q;
            }
            if (value > bestValue) {
                memcpy(&GammaPrime[i * n], alpha, n * sizeof(float));
                pi[i] = a;
                bestValue = value;
            }
        }
    }
    free(alpha);
}

void oracle_pbvi_update(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                        const int *S, const float *T, const float *O, const float *R, const int *Z, const float *B,
                        const float *Gamma, float *GammaPrime, unsigned *pi) {
    oracle_pbvi_update_range(n, ns, m, z, r, rz, gamma, S, T, O, R, Z, B, Gamma, GammaPrime, pi, 0, r);
}

/* Follows pomdp_pbvi_execute_cpu / update_cpu / get_policy_cpu
 * (pomdp_pbvi_cpu.cpp:186-300): horizon steps with the parity swap; the
 * result (GammaOut, piOut) is what get_policy returns. */
void oracle_pbvi_solve(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                       unsigned horizon, const int *S, const float *T, const float *O, const float *R, const int *Z,
                       const float *B, const float *GammaInitial, float *GammaOut, unsigned *piOut) {
    float *G = (float *)malloc(sizeof(float) * r * n);
    float *Gp = (float *)malloc(sizeof(float) * r * n);
    memcpy(G, GammaInitial, sizeof(float) * r * n);
    memcpy(Gp, GammaInitial, sizeof(float) * r * n);
    for (unsigned i = 0; i < r; i++) piOut[i] = 0;
    for (unsigned h = 0; h < horizon; h++) {
        if (h % 2 == 0) oracle_pbvi_update(n, ns, m, z, r, rz, gamma, S, T, O, R, Z, B, G, Gp, piOut);
        else oracle_pbvi_update(n, ns, m, z, r, rz, gamma, S, T, O, R, Z, B, Gp, G, piOut);
    }
    memcpy(GammaOut, (horizon % 2 == 0) ? G : Gp, sizeof(float) * r * n);
    free(G);
    free(Gp);
}

/* ------------------------------------------------------------------------ */
/* PBVI, factored: the same values, projection hoisted out of the belief loop */
/* ------------------------------------------------------------------------ */

/* Proj[j][s] = gamma * sum_l fl(O*T) * Gamma[j][S] for fixed (a, o), exactly
 * the Vtk of pomdp_pbvi_cpu.cpp:66-74 and :89-98 (same operands, same order),
 * so scores built from it are bit-identical to the loop form above. Cost is
 * O(r*n*ns + r*r*rz) per (a, o) instead of O(r*r*rz*ns + n*ns). */
static void project(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned rG, float gamma, const int *S,
                    const float *T, const float *O, const float *Gamma, unsigned a, unsigned o, float *Proj) {
    for (unsigned j = 0; j < rG; j++) {
        const float *g = Gamma + (size_t)j * n;
        float *out = Proj + (size_t)j * n;
        for (unsigned s = 0; s < n; s++) {
            float Vtk = 0.0f;
            for (unsigned l = 0; l < ns; l++) {
                int sp = S[s * m * ns + a * ns + l];
                if (sp < 0) break;
                float ot = O[a * n * z + sp * z + o] * T[s * m * ns + a * ns + l];
                float p = ot * g[sp];
                Vtk = Vtk + p;
            }
            out[s] = Vtk * gamma;
        }
    }
}

/* Bit-identical to oracle_pbvi_update for beliefs [i0, i1); jstarOut
 * (optional, [r][m][z]) receives the chosen alpha per (belief, action, obs). */
void oracle_pbvi_update_factored(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz,
                                 float gamma, const int *S, const float *T, const float *O, const float *R,
                                 const int *Z, const float *B, const float *Gamma, float *GammaPrime, unsigned *pi,
                                 unsigned i0, unsigned i1, unsigned *jstarOut) {
    float *Proj = (float *)malloc(sizeof(float) * (size_t)r * n);
    float *alphaAll = (float *)malloc(sizeof(float) * (size_t)(i1 - i0) * m * n);
    unsigned *jbest = (unsigned *)malloc(sizeof(unsigned) * (size_t)(i1 - i0) * m);
    for (unsigned i = i0; i < i1; i++)
        for (unsigned a = 0; a < m; a++) {
            float *alpha = alphaAll + ((size_t)(i - i0) * m + a) * n;
            for (unsigned s = 0; s < n; s++) alpha[s] = R[s * m + a];
        }
    /* bestj is carried across observations within one (i, a), from 0. */
    for (size_t t = 0; t < (size_t)(i1 - i0) * m; t++) jbest[t] = 0;
    for (unsigned a = 0; a < m; a++) {
        for (unsigned o = 0; o < z; o++) {
            project(n, ns, m, z, r, gamma, S, T, O, Gamma, a, o, Proj);
            for (unsigned i = i0; i < i1; i++) {
                float bestValue = ORACLE_FLT_MIN;
                unsigned bestj = jbest[(size_t)(i - i0) * m + a];
                for (unsigned j = 0; j < r; j++) {
                    const float *pj = Proj + (size_t)j * n;
                    float value = 0.0f;
                    for (unsigned k = 0; k < rz; k++) {
                        int s = Z[i * rz + k];
                        if (s < 0) break;
                        float q = pj[s] * B[i * rz + k];
                        value = value + q;
                    }
                    if (value > bestValue) {
                        bestj = j;
                        bestValue = value;
                    }
                }
                jbest[(size_t)(i - i0) * m + a] = bestj;
                if (jstarOut) jstarOut[((size_t)i * m + a) * z + o] = bestj;
                float *alpha = alphaAll + ((size_t)(i - i0) * m + a) * n;
                const float *pj = Proj + (size_t)bestj * n;
                for (unsigned s = 0; s < n; s++) alpha[s] = alpha[s] + pj[s];
            }
        }
    }
    for (unsigned i = i0; i < i1; i++) {
        float bestValue = ORACLE_FLT_MIN;
        for (unsigned a = 0; a < m; a++) {
            const float *alpha = alphaAll + ((size_t)(i - i0) * m + a) * n;
            float value = 0.0f;
            for (unsigned k = 0; k < rz; k++) {
                int s = Z[i * rz + k];
                if (s < 0) break;
                float q = alpha[s] * B[i * rz + k];
                value = value + q;
            }
            if (value > bestValue) {
                memcpy(&GammaPrime[(size_t)i * n], alpha, n * sizeof(float));
                pi[i] = a;
                bestValue = value;
            }
        }
    }
    free(Proj);
    free(alphaAll);
    free(jbest);
}

/* FP64 restatement of the same backup (factored form, all arithmetic in
 * double, same argmax rules): the reference solution for V(b0) error.
 * Actions are independent until the final action argmax, so they are spread
 * over host threads (each with its own projection buffer). */
typedef struct {
    unsigned n, ns, m, z, r, rz;
    double gamma;
    const int *S;
    const double *T, *O;
    const int *Z;
    const double *B, *Gamma;
    double *alphaAll;
    unsigned a0, astep;
} F64Job;

static void *f64_action_worker(void *arg) {
    const F64Job *J = (const F64Job *)arg;
    const unsigned n = J->n, ns = J->ns, m = J->m, z = J->z, r = J->r, rz = J->rz;
    double *Proj = (double *)malloc(sizeof(double) * (size_t)r * n);
    double *C = (double *)malloc(sizeof(double) * (size_t)n * ns);
    for (unsigned a = J->a0; a < m; a += J->astep) {
        for (unsigned o = 0; o < z; o++) {
            /* C = O(a, s', o) * T(s, a, l), the first product of O*T*Gamma. */
            for (unsigned s = 0; s < n; s++)
                for (unsigned l = 0; l < ns; l++) {
                    int sp = J->S[(size_t)s * m * ns + a * ns + l];
                    C[(size_t)s * ns + l] = sp < 0 ? 0.0
                        : J->O[(size_t)a * n * z + (size_t)sp * z + o] * J->T[(size_t)s * m * ns + a * ns + l];
                }
            for (unsigned j = 0; j < r; j++) {
                const double *g = J->Gamma + (size_t)j * n;
                for (unsigned s = 0; s < n; s++) {
                    const int *Srow = J->S + (size_t)s * m * ns + a * ns;
                    const double *Crow = C + (size_t)s * ns;
                    double v = 0.0;
                    for (unsigned l = 0; l < ns; l++) {
                        int sp = Srow[l];
                        if (sp < 0) break;
                        v += Crow[l] * g[sp];
                    }
                    Proj[(size_t)j * n + s] = v * J->gamma;
                }
            }
            for (unsigned i = 0; i < r; i++) {
                double bestValue = -1e10;
                unsigned bestj = 0;
                for (unsigned j = 0; j < r; j++) {
                    double value = 0.0;
                    for (unsigned k = 0; k < rz; k++) {
                        int s = J->Z[(size_t)i * rz + k];
                        if (s < 0) break;
                        value += Proj[(size_t)j * n + s] * J->B[(size_t)i * rz + k];
                    }
                    if (value > bestValue) { bestj = j; bestValue = value; }
                }
                double *alpha = J->alphaAll + ((size_t)i * m + a) * n;
                for (unsigned s = 0; s < n; s++) alpha[s] += Proj[(size_t)bestj * n + s];
            }
        }
    }
    free(C);
    free(Proj);
    return NULL;
}

void oracle_pbvi_update_f64(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, double gamma,
                            const int *S, const double *T, const double *O, const double *R, const int *Z,
                            const double *B, const double *Gamma, double *GammaPrime, unsigned *pi) {
    double *alphaAll = (double *)malloc(sizeof(double) * (size_t)r * m * n);
    for (unsigned i = 0; i < r; i++)
        for (unsigned a = 0; a < m; a++)
            for (unsigned s = 0; s < n; s++) alphaAll[((size_t)i * m + a) * n + s] = R[(size_t)s * m + a];
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    unsigned nt = (unsigned)(cores < 1 ? 1 : cores);
    if (nt > m) nt = m;
    if (nt > 64) nt = 64;
    F64Job jobs[64];
    pthread_t tid[64];
    for (unsigned t = 0; t < nt; t++) {
        F64Job J = {n, ns, m, z, r, rz, gamma, S, T, O, Z, B, Gamma, alphaAll, t, nt};
        jobs[t] = J;
    }
    unsigned started = 0;
    for (unsigned t = 1; t < nt; t++) {
        if (pthread_create(&tid[t], NULL, f64_action_worker, &jobs[t]) != 0) break;
        started = t;
    }
    f64_action_worker(&jobs[0]);
    for (unsigned t = 1; t <= started; t++) pthread_join(tid[t], NULL);
    /* Actions of threads that failed to start run here. */
    for (unsigned t = started + 1; t < nt; t++) f64_action_worker(&jobs[t]);
    for (unsigned i = 0; i < r; i++) {
        double bestValue = -1e10;
        for (unsigned a = 0; a < m; a++) {
            const double *alpha = alphaAll + ((size_t)i * m + a) * n;
            double value = 0.0;
            for (unsigned k = 0; k < rz; k++) {
                int s = Z[(size_t)i * rz + k];
                if (s < 0) break;
                value += alpha[s] * B[(size_t)i * rz + k];
            }
            if (value > bestValue) {
                memcpy(&GammaPrime[(size_t)i * n], alpha, n * sizeof(double));
                pi[i] = a;
                bestValue = value;
            }
        }
    }
    free(alphaAll);
}

/* ------------------------------------------------------------------------ */
/* V(b) (pomdp_alpha_vectors.cpp:52-79)                                       */
/* ------------------------------------------------------------------------ */

void oracle_alpha_value(unsigned n, unsigned r, const float *Gamma, const unsigned *pi, const float *b, float *Vb,
                        unsigned *a) {
    float best = ORACLE_FLT_MIN;
    unsigned act = 0;
    for (unsigned i = 0; i < r; i++) {
        float V = 0.0f;
        for (unsigned s = 0; s < n; s++) {
            float p = Gamma[i * n + s] * b[s];
            V = V + p;
        }
        if (best < V) {
            best = V;
            act = pi[i];
        }
    }
    *Vb = best;
    *a = act;
}

/* ------------------------------------------------------------------------ */
/* MDP value iteration (mdp_vi_cpu.cpp:36-63, 185-196)                        */
/* ------------------------------------------------------------------------ */

void oracle_mdp_vi_sweep(unsigned n, unsigned ns, unsigned m, float gamma, const int *S, const float *T,
                         const float *R, const float *V, float *VPrime, unsigned *pi) {
    for (unsigned s = 0; s < n; s++) {
        VPrime[s] = -1e+10f;
        for (unsigned a = 0; a < m; a++) {
            float Qsa = R[s * m + a];
            for (unsigned i = 0; i < ns; i++) {
                int sp = S[s * m * ns + a * ns + i];
                if (sp < 0) break;
                float gt = gamma * T[s * m * ns + a * ns + i];
                float p = gt * V[sp];
                Qsa = Qsa + p;
            }
            if (a == 0 || Qsa > VPrime[s]) {
                VPrime[s] = Qsa;
                pi[s] = a;
            }
        }
    }
}

/* Sweeps with the parity swap; V/pi out as mdp_vi_get_policy_cpu returns. */
void oracle_mdp_vi_solve(unsigned n, unsigned ns, unsigned m, float gamma, unsigned horizon, const int *S,
                         const float *T, const float *R, const float *VInitial, float *VOut, unsigned *piOut) {
    float *V = (float *)malloc(sizeof(float) * n);
    float *Vp = (float *)malloc(sizeof(float) * n);
    for (unsigned s = 0; s < n; s++) {
        V[s] = VInitial ? VInitial[s] : 0.0f;
        Vp[s] = V[s];
        piOut[s] = 0;
    }
    for (unsigned h = 0; h < horizon; h++) {
        if (h % 2 == 0) oracle_mdp_vi_sweep(n, ns, m, gamma, S, T, R, V, Vp, piOut);
        else oracle_mdp_vi_sweep(n, ns, m, gamma, S, T, R, Vp, V, piOut);
    }
    memcpy(VOut, (horizon % 2 == 0) ? V : Vp, sizeof(float) * n);
    free(V);
    free(Vp);
}

/* ------------------------------------------------------------------------ */
/* Perseus (pomdp_perseus_cpu.cpp:37-461)                                    */
/* ------------------------------------------------------------------------ */

static float b_dot_alpha(unsigned rz, const int *Z, const float *B, unsigned bIndex, const float *alpha) {
    float acc = 0.0f;
    for (unsigned j = 0; j < rz; j++) {
        int s = Z[bIndex * rz + j];
        if (s < 0) break;
        float p = B[bIndex * rz + j] * alpha[s];
        acc = acc + p;
    }
    return acc;
}

static void compute_Vb(unsigned n, unsigned rz, const int *Z, const float *B, unsigned bIndex, const float *Gamma,
                       unsigned rGamma, float *Vnb, unsigned *idx) {
    *Vnb = ORACLE_FLT_MIN;
    for (unsigned i = 0; i < rGamma; i++) {
        float d = b_dot_alpha(rz, Z, B, bIndex, &Gamma[i * n]);
        if (*Vnb < d) {
            *Vnb = d;
            *idx = i;
        }
    }
}

/* State of one Perseus solve, laid out like POMDPPerseusCPU. */
typedef struct {
    unsigned currentHorizon, rGamma, rGammaPrime, rTilde;
    unsigned *BTilde;
    float *Gamma, *GammaPrime;
    unsigned *pi, *piPrime;
} OraclePerseus;

/* One update (pomdp_perseus_update_cpu). Returns 9 (NOVA_CONVERGED), 0, or
 * 11 (out of memory). With an empty V_n the reference's best-alpha index is
 * unassigned; row 0 is used. */
int oracle_perseus_update(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                          const int *S, const float *T, const float *O, const float *R, const int *Z, const float *B,
                          OraclePerseus *per) {
    float *Gamma, *GammaPrime;
    unsigned *rGamma, *rGammaPrime, *pi, *piPrime;
    if (per->currentHorizon % 2 == 0) {
        Gamma = per->Gamma; GammaPrime = per->GammaPrime; rGamma = &per->rGamma; rGammaPrime = &per->rGammaPrime;
        pi = per->pi; piPrime = per->piPrime;
    } else {
        Gamma = per->GammaPrime; GammaPrime = per->Gamma; rGamma = &per->rGammaPrime; rGammaPrime = &per->rGamma;
        pi = per->piPrime; piPrime = per->pi;
    }
    unsigned bTildeIndex = (unsigned)((float)rand() / (float)RAND_MAX * (float)(per->rTilde));
    if (bTildeIndex >= r) bTildeIndex = r - 1;
    unsigned bIndex = per->BTilde[bTildeIndex];

    /* pomdp_perseus_update_step_cpu (:140-180) */
    float *alpha = (float *)malloc(sizeof(float) * n);
    float *best = (float *)malloc(sizeof(float) * n);
    unsigned alphaAction = 0;
    float bestValue = ORACLE_FLT_MIN;
    unsigned bestjState = 0;
    for (unsigned a = 0; a < m; a++) {
        for (unsigned s = 0; s < n; s++) alpha[s] = R[s * m + a];
        if (*rGamma == 0) {
            /* no alpha to maximise over: add the projection of row 0 */
            for (unsigned o = 0; o < z; o++)
                for (unsigned s = 0; s < n; s++) {
                    float Vtk = 0.0f;
                    for (unsigned l = 0; l < ns; l++) {
                        int sp = S[s * m * ns + a * ns + l];
                        if (sp < 0) break;
                        float ot = O[a * n * z + sp * z + o] * T[s * m * ns + a * ns + l];
                        float p = ot * Gamma[sp];
                        Vtk = Vtk + p;
                    }
                    Vtk = Vtk * gamma;
                    alpha[s] = alpha[s] + Vtk;
                }
        } else {
            pbvi_best_alpha(n, ns, m, z, *rGamma, rz, gamma, S, T, O, Z, B, Gamma, bIndex, a, alpha, &bestjState,
                            NULL);
        }
        float value = b_dot_alpha(rz, Z, B, bIndex, alpha);
        if (value > bestValue) {
            memcpy(best, alpha, n * sizeof(float));
            alphaAction = a;
            bestValue = value;
        }
    }
    float bDotAlpha = b_dot_alpha(rz, Z, B, bIndex, best);
    float Vnb = 0.0f;
    unsigned alphaPrimeIndex = 0;
    compute_Vb(n, rz, Z, B, bIndex, Gamma, *rGamma, &Vnb, &alphaPrimeIndex);
    if (*rGammaPrime + 1 > r) {
        free(alpha); free(best);
        return 11;
    }
    if (bDotAlpha >= Vnb) {
        memcpy(&GammaPrime[(*rGammaPrime) * n], best, n * sizeof(float));
        piPrime[*rGammaPrime] = alphaAction;
    } else {
        memcpy(&GammaPrime[(*rGammaPrime) * n], &Gamma[alphaPrimeIndex * n], n * sizeof(float));
        piPrime[*rGammaPrime] = pi[alphaPrimeIndex];
    }
    (*rGammaPrime)++;
    free(alpha);
    free(best);

    per->rTilde = 0;
    for (unsigned i = 0; i < r; i++) {
        unsigned action = 0;
        float vn = 0.0f, vn1 = 0.0f;
        compute_Vb(n, rz, Z, B, i, Gamma, *rGamma, &vn, &action);
        compute_Vb(n, rz, Z, B, i, GammaPrime, *rGammaPrime, &vn1, &action);
        if (vn1 < vn) per->BTilde[per->rTilde++] = i;
    }
    if (per->rTilde == 0) {
        per->currentHorizon++;
        *rGamma = 0;
        per->rTilde = r;
        for (unsigned i = 0; i < r; i++) per->BTilde[i] = i;
        return 9;
    }
    return 0;
}

/* Full solve (pomdp_perseus_execute_cpu, :222-270). The caller seeds
 * srand() first. Writes the policy rows into GammaOut (capacity r*n) and
 * returns the number of rows, or -1 on error. */
int oracle_perseus_solve(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                         unsigned horizon, const int *S, const float *T, const float *O, const float *R, const int *Z,
                         const float *B, const float *GammaInitial, float *GammaOut, unsigned *piOut) {
    OraclePerseus per;
    per.currentHorizon = 0; per.rGamma = 0; per.rGammaPrime = 0; per.rTilde = r;
    per.BTilde = (unsigned *)malloc(sizeof(unsigned) * r);
    per.Gamma = (float *)malloc(sizeof(float) * r * n);
    per.GammaPrime = (float *)malloc(sizeof(float) * r * n);
    per.pi = (unsigned *)calloc(r, sizeof(unsigned));
    per.piPrime = (unsigned *)calloc(r, sizeof(unsigned));
    memcpy(per.Gamma, GammaInitial, sizeof(float) * r * n);
    memcpy(per.GammaPrime, GammaInitial, sizeof(float) * r * n);
    for (unsigned i = 0; i < r; i++) per.BTilde[i] = i;
    int rows = 0;
    while (per.currentHorizon < horizon) {
        int rc = 0;
        while (rc != 9) {
            rc = oracle_perseus_update(n, ns, m, z, r, rz, gamma, S, T, O, R, Z, B, &per);
            if (rc != 9 && rc != 0) { rows = -1; goto done; }
        }
    }
    if (per.currentHorizon % 2 == 0) {
        rows = (int)per.rGamma;
        memcpy(GammaOut, per.Gamma, sizeof(float) * per.rGamma * n);
        memcpy(piOut, per.pi, sizeof(unsigned) * per.rGamma);
    } else {
        rows = (int)per.rGammaPrime;
        memcpy(GammaOut, per.GammaPrime, sizeof(float) * per.rGammaPrime * n);
        memcpy(piOut, per.piPrime, sizeof(unsigned) * per.rGammaPrime);
    }
done:
    free(per.BTilde); free(per.Gamma); free(per.GammaPrime); free(per.pi); free(per.piPrime);
    return rows;
}

void oracle_srand(unsigned seed) { srand(seed); }

/* One (belief, action) pair of nova's backup in the loop form (the inner
 * body of pomdp_pbvi_update_step_cpu, pomdp_pbvi_cpu.cpp:128-145): fills
 * alphaOut (n) and returns its value at the belief. A belief backup is m of
 * these plus an argmax; the CPU baseline times them in bounded samples. */
float oracle_pbvi_belief_action(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz,
                                float gamma, const int *S, const float *T, const float *O, const float *R,
                                const int *Z, const float *B, const float *Gamma, unsigned i, unsigned a,
                                float *alphaOut) {
    unsigned state = 0;
    for (unsigned s = 0; s < n; s++) alphaOut[s] = R[s * m + a];
    pbvi_best_alpha(n, ns, m, z, r, rz, gamma, S, T, O, Z, B, Gamma, i, a, alphaOut, &state, NULL);
    float value = 0.0f;
    for (unsigned k = 0; k < rz; k++) {
        int s = Z[i * rz + k];
        if (s < 0) break;
        float q = alphaOut[s] * B[i * rz + k];
        value = value + q;
    }
    return value;
}

/* ------------------------------------------------------------------------ */
/* PBVI with recorded selections, FP64 (reference for the GPU adjoint)       */
/* ------------------------------------------------------------------------ */

/* With the selections of each backup held fixed -- act[t][i] (the action
 * whose alpha became Gamma_{t+1}[i]) and sel[t][i][o] (the alpha chosen for
 * observation o) -- a backup of pomdp_pbvi_cpu.cpp:37-162 is
 *   Gamma_{t+1}[i](s) = R(s,a) + sum_o gamma sum_l O(a,S,o) T(s,a,l) Gamma_t[j_o](S),
 * and V(b) = max_i b . Gamma_H[i] (pomdp_alpha_vectors.cpp:52-79, lowest index
 * on ties). Everything here is FP64 and multi-threaded over beliefs. */
typedef struct {
    unsigned n, ns, m, z, r;
    double gamma;
    const int *S;
    const double *T, *O, *R;
    const unsigned *act, *sel; /* this step's [r] and [r][z] */
    const double *Gin;
    double *Gout;
    unsigned i0, i1;
    /* reverse only */
    const double *lam;
    double *lamPrev, *dR, *dT, *dO;
} FixedJob;

static void *fixed_forward_worker(void *arg) {
    const FixedJob *J = (const FixedJob *)arg;
    for (unsigned i = J->i0; i < J->i1; i++) {
        const unsigned a = J->act[i];
        double *out = J->Gout + (size_t)i * J->n;
        for (unsigned s = 0; s < J->n; s++) {
            double v = J->R[(size_t)s * J->m + a];
            for (unsigned o = 0; o < J->z; o++) {
                const double *g = J->Gin + (size_t)J->sel[(size_t)i * J->z + o] * J->n;
                double p = 0.0;
                for (unsigned l = 0; l < J->ns; l++) {
                    const size_t row = ((size_t)s * J->m + a) * J->ns + l;
                    const int sp = J->S[row];
                    if (sp < 0) break;
                    p += J->O[((size_t)a * J->n + sp) * J->z + o] * J->T[row] * g[sp];
                }
                v += J->gamma * p;
            }
            out[s] = v;
        }
    }
    return NULL;
}

static void *fixed_reverse_worker(void *arg) {
    const FixedJob *J = (const FixedJob *)arg;
    for (unsigned i = J->i0; i < J->i1; i++) {
        const unsigned a = J->act[i];
        for (unsigned s = 0; s < J->n; s++) {
            const double lam = J->lam[(size_t)i * J->n + s];
            if (lam == 0.0) continue;
            J->dR[(size_t)s * J->m + a] += lam;
            for (unsigned l = 0; l < J->ns; l++) {
                const size_t row = ((size_t)s * J->m + a) * J->ns + l;
                const int sp = J->S[row];
                if (sp < 0) break;
                const double tv = J->T[row];
                for (unsigned o = 0; o < J->z; o++) {
                    const unsigned j = J->sel[(size_t)i * J->z + o];
                    const double g = J->Gin[(size_t)j * J->n + sp];
                    const size_t oi = ((size_t)a * J->n + sp) * J->z + o;
                    const double ov = J->O[oi];
                    J->dT[row] += J->gamma * lam * ov * g;
                    J->dO[oi] += J->gamma * lam * tv * g;
                    J->lamPrev[(size_t)j * J->n + sp] += J->gamma * lam * tv * ov;
                }
            }
        }
    }
    return NULL;
}

static unsigned oracle_threads(unsigned cap) {
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    unsigned nt = (unsigned)(cores < 1 ? 1 : cores);
    if (nt > cap) nt = cap;
    if (nt > 64) nt = 64;
    return nt < 1 ? 1 : nt;
}

static void run_jobs(FixedJob *jobs, unsigned nt, void *(*fn)(void *)) {
    pthread_t tid[64];
    int started[64] = {0};
    for (unsigned t = 1; t < nt; t++) started[t] = pthread_create(&tid[t], NULL, fn, &jobs[t]) == 0;
    fn(&jobs[0]);
    for (unsigned t = 1; t < nt; t++) {
        if (started[t]) pthread_join(tid[t], NULL);
        else fn(&jobs[t]);
    }
}

/* Forward pass; GammaAll ([H+1][r][n]) receives every Gamma_t. Returns V(b)
 * and the maximising row in *istar; when *istar holds a row index on entry,
 * that row is used instead (the final argmax recorded too). */
double oracle_pbvi_fixed_forward_f64(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, double gamma,
                                     const int *S, const double *T, const double *O, const double *R,
                                     const double *Gamma0, unsigned H, const unsigned *act, const unsigned *sel,
                                     const double *b, unsigned *istar, double *GammaAll) {
    const size_t rn = (size_t)r * n;
    memcpy(GammaAll, Gamma0, rn * sizeof(double));
    const unsigned nt = oracle_threads(r);
    FixedJob jobs[64];
    for (unsigned t = 0; t < H; t++) {
        for (unsigned k = 0; k < nt; k++) {
            FixedJob J;
            memset(&J, 0, sizeof(J));
            J.n = n; J.ns = ns; J.m = m; J.z = z; J.r = r; J.gamma = gamma;
            J.S = S; J.T = T; J.O = O; J.R = R;
            J.act = act + (size_t)t * r; J.sel = sel + (size_t)t * r * z;
            J.Gin = GammaAll + (size_t)t * rn; J.Gout = GammaAll + (size_t)(t + 1) * rn;
            J.i0 = (unsigned)((size_t)r * k / nt); J.i1 = (unsigned)((size_t)r * (k + 1) / nt);
            jobs[k] = J;
        }
        run_jobs(jobs, nt, fixed_forward_worker);
    }
    const double *GH = GammaAll + (size_t)H * rn;
    if (*istar < r) {
        double v = 0.0;
        for (unsigned s = 0; s < n; s++) v += GH[(size_t)*istar * n + s] * b[s];
        return v;
    }
    double best = -1e10;
    unsigned bi = 0xffffffffu;
    for (unsigned i = 0; i < r; i++) {
        double v = 0.0;
        for (unsigned s = 0; s < n; s++) v += GH[(size_t)i * n + s] * b[s];
        if (v > best) { best = v; bi = i; }
    }
    *istar = bi;
    return best;
}

/* Reverse pass (direct form, every (i, s, l, o) term): gradients of V(b) with
 * respect to R [n][m], T [n][m][ns], O [m][n][z] and Gamma0 [r][n]. A row
 * index in istarFixed fixes the final argmax (0xffffffff: take the FP64 one). */
double oracle_pbvi_fixed_reverse_f64(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, double gamma,
                                     const int *S, const double *T, const double *O, const double *R,
                                     const double *Gamma0, unsigned H, const unsigned *act, const unsigned *sel,
                                     const double *b, unsigned istarFixed, double *dR, double *dT, double *dO,
                                     double *dGamma0) {
    const size_t rn = (size_t)r * n;
    double *GammaAll = (double *)malloc(sizeof(double) * (size_t)(H + 1) * rn);
    unsigned istar = istarFixed;
    const double V = oracle_pbvi_fixed_forward_f64(n, ns, m, z, r, gamma, S, T, O, R, Gamma0, H, act, sel, b,
                                                   &istar, GammaAll);
    const size_t nR = (size_t)n * m, nT = (size_t)n * m * ns, nO = (size_t)m * n * z;
    memset(dR, 0, nR * sizeof(double));
    memset(dT, 0, nT * sizeof(double));
    memset(dO, 0, nO * sizeof(double));
    double *lam = (double *)calloc(rn, sizeof(double));
    if (istar != 0xffffffffu) memcpy(lam + (size_t)istar * n, b, n * sizeof(double));
    const unsigned nt = oracle_threads(r);
    /* Per-thread accumulators, summed after every step. */
    double *acc = (double *)malloc(sizeof(double) * (size_t)nt * (rn + nR + nT + nO));
    FixedJob jobs[64];
    for (unsigned t = H; t >= 1; t--) {
        memset(acc, 0, sizeof(double) * (size_t)nt * (rn + nR + nT + nO));
        for (unsigned k = 0; k < nt; k++) {
            double *base = acc + (size_t)k * (rn + nR + nT + nO);
            FixedJob J;
            memset(&J, 0, sizeof(J));
            J.n = n; J.ns = ns; J.m = m; J.z = z; J.r = r; J.gamma = gamma;
            J.S = S; J.T = T; J.O = O; J.R = R;
            J.act = act + (size_t)(t - 1) * r; J.sel = sel + (size_t)(t - 1) * r * z;
            J.Gin = GammaAll + (size_t)(t - 1) * rn;
            J.i0 = (unsigned)((size_t)r * k / nt); J.i1 = (unsigned)((size_t)r * (k + 1) / nt);
            J.lam = lam;
            J.lamPrev = base; J.dR = base + rn; J.dT = base + rn + nR; J.dO = base + rn + nR + nT;
            jobs[k] = J;
        }
        run_jobs(jobs, nt, fixed_reverse_worker);
        memset(lam, 0, rn * sizeof(double));
        for (unsigned k = 0; k < nt; k++) {
            const double *base = acc + (size_t)k * (rn + nR + nT + nO);
            for (size_t e = 0; e < rn; e++) lam[e] += base[e];
            for (size_t e = 0; e < nR; e++) dR[e] += base[rn + e];
            for (size_t e = 0; e < nT; e++) dT[e] += base[rn + nR + e];
            for (size_t e = 0; e < nO; e++) dO[e] += base[rn + nR + nT + e];
        }
    }
    if (dGamma0) memcpy(dGamma0, lam, rn * sizeof(double));
    free(acc);
    free(lam);
    free(GammaAll);
    return V;
}

/* ------------------------------------------------------------------------ */
/* Belief expansion (pomdp_expand_cpu.cpp, pomdp_expand_gpu.cu)              */
/* ------------------------------------------------------------------------ */

#define ORACLE_FLT_MAX (1e+10f)    /* nova's FLT_MAX, include/nova/constants.h:33 */

/* pomdp_expand_construct_belief_cpu, pomdp_expand_cpu.cpp:39-53 */
static void construct_belief(unsigned n, unsigned rz, const int *Z, const float *B, unsigned i, float *b) {
    for (unsigned s = 0; s < n; s++) b[s] = 0.0f;
    for (unsigned j = 0; j < rz; j++) {
        int s = Z[(size_t)i * rz + j];
        if (s < 0) break;
        b[s] = B[(size_t)i * rz + j];
    }
}

/* pomdp_belief_update_cpu, pomdp_model_cpu.cpp:89-137. Returns 0, or 1 when
 * the normaliser is below FLT_ERR_TOL (bp then holds the unnormalised values). */
int oracle_belief_update(unsigned n, unsigned ns, unsigned m, unsigned z, const int *S, const float *T,
                         const float *O, const float *b, unsigned a, unsigned o, float *bp) {
    for (unsigned sp = 0; sp < n; sp++) bp[sp] = 0.0f;
    for (unsigned s = 0; s < n; s++) {
        for (unsigned i = 0; i < ns; i++) {
            int sp = S[(size_t)s * m * ns + a * ns + i];
            if (sp < 0) break;
            float t = T[(size_t)s * m * ns + a * ns + i] * b[s];
            bp[sp] = bp[sp] + t;
        }
    }
    float norm = 0.0f;
    for (unsigned sp = 0; sp < n; sp++) {
        bp[sp] = bp[sp] * O[(size_t)a * n * z + (size_t)sp * z + o];
        norm = norm + bp[sp];
    }
    if (fabs((double)fabsf(norm)) < 1e-9) return 1;
    for (unsigned sp = 0; sp < n; sp++) bp[sp] = bp[sp] / norm;
    return 0;
}

/* pomdp_expand_probability_observation_cpu, pomdp_expand_cpu.cpp:56-78 */
static float prob_obs(unsigned n, unsigned ns, unsigned m, unsigned z, const int *S, const float *T,
                      const float *O, const float *b, unsigned a, unsigned o) {
    float pr = 0.0f;
    for (unsigned s = 0; s < n; s++) {
        float val = 0.0f;
        for (unsigned i = 0; i < ns; i++) {
            int sp = S[(size_t)s * m * ns + a * ns + i];
            if (sp < 0) break;
            float t = T[(size_t)s * m * ns + a * ns + i] * O[(size_t)a * n * z + (size_t)sp * z + o];
            val = val + t;
        }
        float q = val * b[s];
        pr = pr + q;
    }
    return pr;
}

static unsigned draw(float scale) {
    return (unsigned)((float)rand() / (float)RAND_MAX * scale);
}

/* pomdp_expand_random_cpu, pomdp_expand_cpu.cpp:81-150, after srand(seed)
 * (the reference seeds with time(nullptr)). Bnew [num][n]. */
void oracle_expand_random(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, unsigned horizon,
                          const int *S, const float *T, const float *O, const int *Z, const float *B, unsigned num,
                          unsigned seed, float *Bnew) {
    srand(seed);
    float *b = (float *)malloc(sizeof(float) * n);
    float *bp = (float *)malloc(sizeof(float) * n);
    for (size_t k = 0; k < (size_t)num * n; k++) Bnew[k] = 0.0f;
    unsigned i = 0;
    while (i < num) {
        unsigned b0 = draw((float)r);
        construct_belief(n, rz, Z, B, b0, b);
        unsigned h = draw((float)(horizon + 1));
        for (unsigned t = 0; t < h; t++) {
            unsigned a = draw((float)m);
            float cur = 0.0f;
            float target = (float)rand() / (float)RAND_MAX;
            unsigned o = 0;
            for (unsigned op = 0; op < z; op++) {
                float pr = prob_obs(n, ns, m, z, S, T, O, b, a, op);
                cur = cur + pr;
                if (cur >= target && pr > 0.0f) { o = op; break; }
            }
            oracle_belief_update(n, ns, m, z, S, T, O, b, a, o, bp);
            memcpy(b, bp, sizeof(float) * n);
            memcpy(Bnew + (size_t)i * n, b, sizeof(float) * n);
            i++;
            if (i >= num) break;
        }
    }
    free(b);
    free(bp);
}

/* pomdp_expand_random_gpu, pomdp_expand_gpu.cu:127-215, after srand(seed):
 * starts every trajectory at belief 0, which is also Bnew[0]; returns the
 * maximum non-zero count over the expanded beliefs (rows 1..). */
unsigned oracle_expand_random_from_b0(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned rz, unsigned horizon,
                                      const int *S, const float *T, const float *O, const int *Z, const float *B,
                                      unsigned num, unsigned seed, float *Bnew) {
    srand(seed);
    unsigned maxNZ = 0;
    float *b0 = (float *)malloc(sizeof(float) * n);
    float *b = (float *)malloc(sizeof(float) * n);
    float *bp = (float *)malloc(sizeof(float) * n);
    construct_belief(n, rz, Z, B, 0, b0);
    memcpy(Bnew, b0, sizeof(float) * n);
    unsigned i = 1;
    while (i < num) {
        unsigned h = draw((float)(horizon + 1));
        memcpy(b, b0, sizeof(float) * n);
        for (unsigned t = 0; t < h; t++) {
            unsigned a = draw((float)m);
            float cur = 0.0f;
            float target = (float)rand() / (float)RAND_MAX;
            unsigned o = 0;
            for (unsigned op = 0; op < z; op++) {
                float pr = prob_obs(n, ns, m, z, S, T, O, b, a, op);
                cur = cur + pr;
                if (cur >= target) { o = op; break; }
            }
            oracle_belief_update(n, ns, m, z, S, T, O, b, a, o, bp);
            memcpy(b, bp, sizeof(float) * n);
            unsigned nz = 0;
            for (unsigned s = 0; s < n; s++) nz += b[s] > 0.0f ? 1u : 0u;
            if (nz > maxNZ) maxNZ = nz;
            memcpy(Bnew + (size_t)i * n, b, sizeof(float) * n);
            i++;
            if (i >= num) break;
        }
    }
    free(b0);
    free(b);
    free(bp);
    return maxNZ;
}

/* pomdp_expand_distinct_beliefs_cpu, pomdp_expand_cpu.cpp:153-241. Bnew
 * [r][n]; a belief with no valid (a, o) gets a zero row (the reference
 * copies an uninitialised buffer). */
void oracle_expand_distinct_range(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz,
                                  const int *S, const float *T, const float *O, const int *Z, const float *B,
                                  unsigned i0, unsigned i1, float *Bnew) {
    float *b = (float *)malloc(sizeof(float) * n);
    float *bp = (float *)malloc(sizeof(float) * n);
    float *btmp = (float *)malloc(sizeof(float) * n);
    for (unsigned i = i0; i < i1; i++) {
        construct_belief(n, rz, Z, B, i, b);
        float *star = Bnew + (size_t)i * n;
        for (unsigned s = 0; s < n; s++) star[s] = 0.0f;
        float starValue = ORACLE_FLT_MIN;
        for (unsigned a = 0; a < m; a++) {
            for (unsigned o = 0; o < z; o++) {
                float pr = prob_obs(n, ns, m, z, S, T, O, b, a, o);
                if (pr == 0.0f) continue;
                if (oracle_belief_update(n, ns, m, z, S, T, O, b, a, o, bp) != 0) continue;
                float jStar = ORACLE_FLT_MAX;
                for (unsigned j = 0; j < r; j++) {
                    construct_belief(n, rz, Z, B, j, btmp);
                    float d = 0.0f;
                    for (unsigned s = 0; s < n; s++) d = d + fabsf(btmp[s] - bp[s]);
                    if (d < jStar) jStar = d;
                }
                if (jStar > starValue) {
                    memcpy(star, bp, sizeof(float) * n);
                    starValue = jStar;
                }
            }
        }
    }
    free(b);
    free(bp);
    free(btmp);
}

void oracle_expand_distinct(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, const int *S,
                            const float *T, const float *O, const int *Z, const float *B, float *Bnew) {
    oracle_expand_distinct_range(n, ns, m, z, r, rz, S, T, O, Z, B, 0, r, Bnew);
}

/* pomdp_expand_pema_cpu, pomdp_expand_cpu.cpp:244-383 (policy Gamma [pr][n]).
 * Bnew [n] (one belief). */
void oracle_expand_pema(unsigned n, unsigned ns, unsigned m, unsigned z, unsigned r, unsigned rz, float gamma,
                        const int *S, const float *T, const float *O, const float *R, const int *Z, const float *B,
                        unsigned pr, const float *Gamma, float *Bnew) {
    for (unsigned s = 0; s < n; s++) Bnew[s] = 0.0f;
    float bStar = ORACLE_FLT_MIN;
    float Rmax = ORACLE_FLT_MIN, Rmin = ORACLE_FLT_MAX;
    for (unsigned s = 0; s < n; s++)
        for (unsigned a = 0; a < m; a++) {
            float v = R[(size_t)s * m + a];
            if (Rmax < v) Rmax = v;
            if (Rmin > v) Rmin = v;
        }
    float *b = (float *)malloc(sizeof(float) * n);
    float *bp = (float *)malloc(sizeof(float) * n);
    float *bc = (float *)malloc(sizeof(float) * n);
    float *bt = (float *)malloc(sizeof(float) * n);
    unsigned *oStar = (unsigned *)malloc(sizeof(unsigned) * m);
    float *oStarValue = (float *)malloc(sizeof(float) * m);
    const float hi = Rmax / (1.0f - gamma), lo = Rmin / (1.0f - gamma);
    for (unsigned i = 0; i < r; i++) {
        unsigned aStar = 0;
        float aStarValue = ORACLE_FLT_MIN;
        construct_belief(n, rz, Z, B, i, b);
        for (unsigned a = 0; a < m; a++) { oStar[a] = 0; oStarValue[a] = ORACLE_FLT_MIN; }
        for (unsigned a = 0; a < m; a++) {
            float aValue = 0.0f;
            for (unsigned o = 0; o < z; o++) {
                float p = 0.0f;
                for (unsigned j = 0; j < rz; j++) {
                    int s = Z[(size_t)i * rz + j];
                    if (s < 0) break;
                    for (unsigned k = 0; k < ns; k++) {
                        int sp = S[(size_t)s * m * ns + a * ns + k];
                        if (sp < 0) break;
                        float t1 = T[(size_t)s * m * ns + a * ns + k] * O[(size_t)a * n * z + (size_t)sp * z + o];
                        float t2 = t1 * B[(size_t)i * rz + j];
                        p = p + t2;
                    }
                }
                if (oracle_belief_update(n, ns, m, z, S, T, O, b, a, o, bp) != 0) continue;
                float best = ORACLE_FLT_MAX;
                for (unsigned j = 0; j < r; j++) {
                    construct_belief(n, rz, Z, B, j, bt);
                    float d = 0.0f;
                    for (unsigned s = 0; s < n; s++) d = d + fabsf(bp[s] - bt[s]);
                    if (d < best) { memcpy(bc, bt, sizeof(float) * n); best = d; }
                }
                unsigned alphaStar = 0;
                for (unsigned j = 0; j < pr; j++)
                    for (unsigned s = 0; s < n; s++) {
                        float Vb = Gamma[(size_t)j * n + s] * bc[s];
                        if (Vb < ORACLE_FLT_MIN) alphaStar = j;
                    }
                float eps = 0.0f;
                for (unsigned s = 0; s < n; s++) {
                    float d = bp[s] - bc[s];
                    float c = (bp[s] >= b[s] ? hi : lo) - Gamma[(size_t)alphaStar * n + s];
                    float t = c * d;
                    eps = eps + t;
                }
                float v = p * eps;
                if (v > oStarValue[a]) { oStar[a] = o; oStarValue[a] = v; }
                aValue = aValue + v;
            }
            if (aValue > aStarValue) { aStar = a; aStarValue = aValue; }
        }
        if (aStarValue > bStar) {
            if (oracle_belief_update(n, ns, m, z, S, T, O, b, aStar, oStar[aStar], bp) == 0)
                memcpy(Bnew, bp, sizeof(float) * n);
            else
                memcpy(Bnew, b, sizeof(float) * n);
            bStar = aStarValue;
        }
    }
    free(b); free(bp); free(bc); free(bt); free(oStar); free(oStarValue);
}
