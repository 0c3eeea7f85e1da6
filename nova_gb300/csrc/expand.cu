// nova-gb300: belief-set expansion on the GB300.
//
// Replaces pomdp_expand_random_cpu, pomdp_expand_distinct_beliefs_cpu and
// pomdp_expand_pema_cpu (pomdp_expand_cpu.cpp:81-383) and
// pomdp_expand_random_gpu (pomdp_expand_gpu.cu:127-215), with the
// reference's FP32 operation order throughout, so the new beliefs are
// bit-identical:
//
//   * belief update b'(s') = O(a,s',o) * sum_{(s,i): S(s,a,i)=s'} T(s,a,i) b(s),
//     then normalised (pomdp_model_cpu.cpp:89-137). The reference scatters
//     over (s, i) in order; here each s' gathers its predecessors from a
//     per-action list sorted by (s, i), which adds the same terms in the same
//     order, so the states s' run in parallel.
//   * every sum the reference accumulates sequentially over s (observation
//     probabilities, normalisers, L1 distances, error bounds) is formed the
//     same way: the terms are computed in parallel and one thread adds them in
//     order.
//   * one block per belief (distinct, PEMA) or per trajectory (random); the
//     L1 distances to all r beliefs run one belief per thread over a dense,
//     state-major copy of B.
//
// The random expansions draw from libc rand() on the host exactly as the
// reference does (srand(time(nullptr)), or a fixed seed set with
// nova_gb300_expand_seed); the draws do not depend on belief values, so the
// host lays out every trajectory first and the device runs them in parallel.

#include "common.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <ctime>
#include <vector>

#include <nova/constants.h>
#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>
#include <nova/pomdp/utilities/pomdp_model_cpu.h>
#include <nova/pomdp/utilities/pomdp_expand_cpu.h>
#include <nova/pomdp/utilities/pomdp_expand_gpu.h>
#include <nova/pomdp/utilities/pomdp_sigma_cpu.h>
#include <nova/nova_gb300.h>

using nova::POMDP;
using nova::POMDPAlphaVectors;

namespace nova_gb300 {
namespace {

constexpr unsigned kThreads = 256;
constexpr unsigned kNoIndex = 0xffffffffu;

std::atomic<unsigned> g_seed_fixed{0};
std::atomic<unsigned> g_seed{0};

void seed_rand() {
    if (g_seed_fixed.load()) srand(g_seed.load());
    else srand((unsigned)time(nullptr));
}

unsigned draw(float scale) { return (unsigned)((float)rand() / (float)RAND_MAX * scale); }

struct ExpModel {
    unsigned n, ns, m, z, r, rz;
    float gamma;
    const int *S;
    const float *T, *O, *R;
    const int *Z;
    const float *B;
    const unsigned *predStart;  // [m][n+1]
    const unsigned *predIdx;    // entries (s*m + a)*ns + i, sorted by (s, i) per (a, s')
    const float *BT;            // [n][r] dense beliefs, state-major
};

// Shared-memory layout of one block: b, bp, aux, tmp (n floats each) plus
// scalars.
struct BlockBufs {
    float *b, *bp, *aux, *tmp;
};

// Thread 0 adds v[0..n) in order; the result is returned to every thread.
__device__ float seq_sum(const float *v, unsigned n, float *slot) {
    __syncthreads();
    if (threadIdx.x == 0) {
        float acc = 0.0f;
        for (unsigned s = 0; s < n; s++) acc = fadd(acc, v[s]);
        *slot = acc;
    }
    __syncthreads();
    return *slot;
}

// pomdp_expand_probability_observation_cpu (pomdp_expand_cpu.cpp:56-78).
__device__ float prob_obs_dense(const ExpModel &md, const float *b, float *tmp, unsigned a, unsigned o, float *slot) {
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        const size_t row = ((size_t)s * md.m + a) * md.ns;
        float val = 0.0f;
        for (unsigned i = 0; i < md.ns; i++) {
            const int sp = md.S[row + i];
            if (sp < 0) break;
            val = fadd(val, fmul(md.T[row + i], md.O[((size_t)a * md.n + sp) * md.z + o]));
        }
        tmp[s] = fmul(val, b[s]);
    }
    return seq_sum(tmp, md.n, slot);
}

// pomdp_belief_update_cpu (pomdp_model_cpu.cpp:89-137). Returns true when
// the normaliser reaches FLT_ERR_TOL; otherwise bp keeps the unnormalised
// values, as the reference's does.
__device__ bool belief_update(const ExpModel &md, const float *b, float *bp, unsigned a, unsigned o, float *slot) {
    for (unsigned sp = threadIdx.x; sp < md.n; sp += blockDim.x) {
        const unsigned e0 = md.predStart[(size_t)a * (md.n + 1) + sp];
        const unsigned e1 = md.predStart[(size_t)a * (md.n + 1) + sp + 1];
        float v = 0.0f;
        for (unsigned k = e0; k < e1; k++) {
            const unsigned e = md.predIdx[k];
            const unsigned s = e / (md.m * md.ns);
            v = fadd(v, fmul(md.T[e], b[s]));
        }
        bp[sp] = fmul(v, md.O[((size_t)a * md.n + sp) * md.z + o]);
    }
    const float norm = seq_sum(bp, md.n, slot);
    if (fabs((double)fabsf(norm)) < NOVA_FLT_ERR_TOL) return false;
    for (unsigned sp = threadIdx.x; sp < md.n; sp += blockDim.x) bp[sp] = __fdiv_rn(bp[sp], norm);
    __syncthreads();
    return true;
}

__device__ void load_belief(const ExpModel &md, unsigned i, float *b) {
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) b[s] = md.BT[(size_t)s * md.r + i];
    __syncthreads();
}

// L1 distance sum_s |b_j(s) - bp(s)| in state order, one belief j per thread;
// returns the smallest and (in *argOut) the lowest j attaining it.
__device__ float min_distance(const ExpModel &md, const float *bp, unsigned *argOut, float *sv, unsigned *si) {
    float best = NOVA_FLT_MAX;
    unsigned bj = kNoIndex;
    for (unsigned j = threadIdx.x; j < md.r; j += blockDim.x) {
        float d = 0.0f;
        for (unsigned s = 0; s < md.n; s++) d = fadd(d, fabsf(__fsub_rn(md.BT[(size_t)s * md.r + j], bp[s])));
        if (d < best) { best = d; bj = j; }
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bj;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned t = 1; t < blockDim.x; t++) {
            if (si[t] == kNoIndex) continue;
            if (si[0] == kNoIndex || sv[t] < sv[0] || (sv[t] == sv[0] && si[t] < si[0])) { sv[0] = sv[t]; si[0] = si[t]; }
        }
    }
    __syncthreads();
    const float v = sv[0];
    if (argOut) *argOut = si[0];
    __syncthreads();
    return v;
}

__device__ BlockBufs carve(float *smem, unsigned n) {
    return BlockBufs{smem, smem + n, smem + 2 * (size_t)n, smem + 3 * (size_t)n};
}

// pomdp_expand_distinct_beliefs_cpu (pomdp_expand_cpu.cpp:153-241): for
// belief i, the successor b'(b_i, a, o) farthest (in min L1 distance) from
// the belief set. One block per belief.
__global__ void __launch_bounds__(kThreads) distinct_kernel(ExpModel md, float *__restrict__ Bnew) {
    extern __shared__ __align__(16) float smem[];
    __shared__ float slot, sv[kThreads];
    __shared__ unsigned si[kThreads];
    __shared__ int take;
    BlockBufs w = carve(smem, md.n);
    float *star = w.aux;
    const unsigned i = blockIdx.x;
    load_belief(md, i, w.b);
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) star[s] = 0.0f;
    float starValue = NOVA_FLT_MIN;
    for (unsigned a = 0; a < md.m; a++) {
        for (unsigned o = 0; o < md.z; o++) {
            const float pr = prob_obs_dense(md, w.b, w.tmp, a, o, &slot);
            if (pr == 0.0f) continue;
            if (!belief_update(md, w.b, w.bp, a, o, &slot)) continue;
            const float jStar = min_distance(md, w.bp, nullptr, sv, si);
            if (threadIdx.x == 0) take = jStar > starValue ? 1 : 0;
            __syncthreads();
            if (take) {
                starValue = jStar;
                for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) star[s] = w.bp[s];
            }
            __syncthreads();
        }
    }
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) Bnew[(size_t)i * md.n + s] = star[s];
}

// One step of a random trajectory, laid out by the host.
struct Step {
    unsigned traj;      // trajectory
    unsigned a;         // action drawn
    float target;       // observation draw in [0, 1]
    unsigned out;       // row of Bnew written after the step
};

// Trajectory k starts from belief start[k] and runs steps [first[k], first[k+1]).
// checkPositive: the CPU form also requires Pr(o) > 0 for the chosen o.
__global__ void __launch_bounds__(kThreads) random_kernel(ExpModel md, const unsigned *__restrict__ start,
                                                          const unsigned *__restrict__ first,
                                                          const Step *__restrict__ steps, int checkPositive,
                                                          float *__restrict__ Bnew) {
    extern __shared__ __align__(16) float smem[];
    __shared__ float slot;
    __shared__ unsigned chosen;
    BlockBufs w = carve(smem, md.n);
    const unsigned k = blockIdx.x;
    load_belief(md, start[k], w.b);
    for (unsigned q = first[k]; q < first[k + 1]; q++) {
        const Step st = steps[q];
        float cur = 0.0f;
        if (threadIdx.x == 0) chosen = 0;
        for (unsigned op = 0; op < md.z; op++) {
            const float pr = prob_obs_dense(md, w.b, w.tmp, st.a, op, &slot);
            cur = fadd(cur, pr);
            if (cur >= st.target && (!checkPositive || pr > 0.0f)) {
                if (threadIdx.x == 0) chosen = op;
                break;
            }
        }
        __syncthreads();
        belief_update(md, w.b, w.bp, st.a, chosen, &slot);
        __syncthreads();
        for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
            w.b[s] = w.bp[s];
            Bnew[(size_t)st.out * md.n + s] = w.bp[s];
        }
        __syncthreads();
    }
}

// pomdp_expand_pema_cpu (pomdp_expand_cpu.cpp:244-383), per belief i: the
// best action's error bound and its (action, observation).
__global__ void __launch_bounds__(kThreads) pema_kernel(ExpModel md, unsigned pr, const float *__restrict__ Gamma,
                                                        float *__restrict__ aStarValueOut,
                                                        unsigned *__restrict__ aStarOut,
                                                        unsigned *__restrict__ oStarOut) {
    extern __shared__ __align__(16) float smem[];
    __shared__ float slot, sv[kThreads];
    __shared__ unsigned si[kThreads];
    __shared__ unsigned alphaStar, closest;
    BlockBufs w = carve(smem, md.n);
    const unsigned i = blockIdx.x;
    load_belief(md, i, w.b);
    // Rmax / (1 - gamma) and Rmin / (1 - gamma) from the reward range.
    if (threadIdx.x == 0) {
        float Rmax = NOVA_FLT_MIN, Rmin = NOVA_FLT_MAX;
        for (unsigned s = 0; s < md.n; s++)
            for (unsigned a = 0; a < md.m; a++) {
                const float v = md.R[(size_t)s * md.m + a];
                if (Rmax < v) Rmax = v;
                if (Rmin > v) Rmin = v;
            }
        sv[0] = __fdiv_rn(Rmax, __fsub_rn(1.0f, md.gamma));
        sv[1] = __fdiv_rn(Rmin, __fsub_rn(1.0f, md.gamma));
    }
    __syncthreads();
    const float hi = sv[0], lo = sv[1];
    __syncthreads();
    unsigned aStar = 0;
    float aStarValue = NOVA_FLT_MIN;
    unsigned oStarBest = 0;
    for (unsigned a = 0; a < md.m; a++) {
        float aValue = 0.0f;
        unsigned oStar = 0;
        float oStarValue = NOVA_FLT_MIN;
        for (unsigned o = 0; o < md.z; o++) {
            // Pr(o | b, a) over the belief's support, in (support, successor) order.
            if (threadIdx.x == 0) {
                float p = 0.0f;
                for (unsigned j = 0; j < md.rz; j++) {
                    const int s = md.Z[(size_t)i * md.rz + j];
                    if (s < 0) break;
                    const size_t row = ((size_t)s * md.m + a) * md.ns;
                    for (unsigned q = 0; q < md.ns; q++) {
                        const int sp = md.S[row + q];
                        if (sp < 0) break;
                        p = fadd(p, fmul(fmul(md.T[row + q], md.O[((size_t)a * md.n + sp) * md.z + o]),
                                         md.B[(size_t)i * md.rz + j]));
                    }
                }
                slot = p;
            }
            __syncthreads();
            const float p = slot;
            __syncthreads();
            if (!belief_update(md, w.b, w.bp, a, o, &slot)) continue;
            min_distance(md, w.bp, &closest, sv, si);
            float *bc = w.aux;
            for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) bc[s] = md.BT[(size_t)s * md.r + closest];
            // The reference's alpha search keeps the last j with some
            // Gamma_j(s) * bc(s) below -1e10 (its running value never moves).
            if (threadIdx.x == 0) alphaStar = 0;
            __syncthreads();
            for (unsigned j = threadIdx.x; j < pr; j += blockDim.x) {
                bool hit = false;
                for (unsigned s = 0; s < md.n && !hit; s++) hit = fmul(Gamma[(size_t)j * md.n + s], bc[s]) < NOVA_FLT_MIN;
                if (hit) atomicMax(&alphaStar, j);
            }
            __syncthreads();
            const float *g = Gamma + (size_t)alphaStar * md.n;
            for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
                const float c = __fsub_rn(w.bp[s] >= w.b[s] ? hi : lo, g[s]);
                w.tmp[s] = fmul(c, __fsub_rn(w.bp[s], bc[s]));
            }
            const float eps = seq_sum(w.tmp, md.n, &slot);
            const float v = fmul(p, eps);
            if (v > oStarValue) { oStar = o; oStarValue = v; }
            aValue = fadd(aValue, v);
        }
        if (aValue > aStarValue) { aStar = a; aStarValue = aValue; oStarBest = oStar; }
    }
    if (threadIdx.x == 0) {
        aStarValueOut[i] = aStarValue;
        aStarOut[i] = aStar;
        oStarOut[i] = oStarBest;
    }
}

// b'(b_i, a, o), or b_i itself when the update is invalid (PEMA's final step).
__global__ void __launch_bounds__(kThreads) update_one_kernel(ExpModel md, unsigned i, unsigned a, unsigned o,
                                                              float *__restrict__ out) {
    extern __shared__ __align__(16) float smem[];
    __shared__ float slot;
    BlockBufs w = carve(smem, md.n);
    load_belief(md, i, w.b);
    const bool ok = belief_update(md, w.b, w.bp, a, o, &slot);
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) out[s] = ok ? w.bp[s] : w.b[s];
}

__global__ void dense_beliefs_kernel(unsigned n, unsigned r, unsigned rz, const int *__restrict__ Z,
                                     const float *__restrict__ B, float *__restrict__ BT) {
    const unsigned i = blockIdx.x;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) BT[(size_t)s * r + i] = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned j = 0; j < rz; j++) {
            const int s = Z[(size_t)i * rz + j];
            if (s < 0) break;
            BT[(size_t)s * r + i] = B[(size_t)i * rz + j];
        }
    }
}

// Device copies of a host-array POMDP plus the predecessor lists and the
// dense beliefs, freed on destruction.
struct ExpWorkspace {
    ExpModel md{};
    int *S = nullptr, *Z = nullptr;
    float *T = nullptr, *O = nullptr, *R = nullptr, *B = nullptr, *BT = nullptr;
    unsigned *predStart = nullptr, *predIdx = nullptr;
    size_t smem = 0;
    ~ExpWorkspace() {
        cudaFree(S); cudaFree(Z); cudaFree(T); cudaFree(O); cudaFree(R); cudaFree(B); cudaFree(BT);
        cudaFree(predStart); cudaFree(predIdx);
    }
};

int build_workspace(const POMDP *p, ExpWorkspace &ws, const char *fn) {
    const unsigned n = p->n, ns = p->ns, m = p->m, z = p->z, r = p->r, rz = p->rz;
    const size_t nms = (size_t)n * m * ns;
    int rc;
    // Predecessors of each (a, s'), in (s, i) order: action a's lists are
    // start[a*(n+1) + s'] .. start[a*(n+1) + s' + 1] of one global array.
    std::vector<unsigned> count((size_t)m * n, 0u), start((size_t)m * (n + 1), 0u), idx(std::max<size_t>(nms, 1));
    for (unsigned s = 0; s < n; s++)
        for (unsigned a = 0; a < m; a++)
            for (unsigned i = 0; i < ns; i++) {
                const int sp = p->S[((size_t)s * m + a) * ns + i];
                if (sp < 0) break;
                if ((unsigned)sp >= n) {
                    NOVA_ERR(fn, "Invalid arguments: a successor state is out of range.");
                    return NOVA_ERROR_INVALID_DATA;
                }
                count[(size_t)a * n + sp]++;
            }
    unsigned running = 0;
    for (unsigned a = 0; a < m; a++) {
        for (unsigned sp = 0; sp < n; sp++) {
            start[(size_t)a * (n + 1) + sp] = running;
            running += count[(size_t)a * n + sp];
        }
        start[(size_t)a * (n + 1) + n] = running;
    }
    std::vector<unsigned> cursor(start);
    for (unsigned s = 0; s < n; s++)
        for (unsigned a = 0; a < m; a++)
            for (unsigned i = 0; i < ns; i++) {
                const int sp = p->S[((size_t)s * m + a) * ns + i];
                if (sp < 0) break;
                idx[cursor[(size_t)a * (n + 1) + sp]++] = (unsigned)(((size_t)s * m + a) * ns + i);
            }
    if ((rc = dev_alloc(&ws.S, nms, fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.T, nms, fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.O, (size_t)m * n * z, fn, "the observation transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.R, (size_t)n * m, fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.Z, (size_t)r * rz, fn, "the belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.B, (size_t)r * rz, fn, "the belief values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.BT, (size_t)n * r, fn, "the dense beliefs")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.predStart, start.size(), fn, "the predecessor offsets")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws.predIdx, std::max<size_t>(nms, 1), fn, "the predecessors")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.S, p->S, nms * sizeof(int), fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.T, p->T, nms * sizeof(float), fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.O, p->O, (size_t)m * n * z * sizeof(float), fn, "the observation transitions")) != NOVA_SUCCESS)
        return rc;
    if ((rc = h2d(ws.R, p->R, (size_t)n * m * sizeof(float), fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.Z, p->Z, (size_t)r * rz * sizeof(int), fn, "the belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.B, p->B, (size_t)r * rz * sizeof(float), fn, "the belief values")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws.predStart, start.data(), start.size() * sizeof(unsigned), fn, "the predecessor offsets")) !=
            NOVA_SUCCESS)
        return rc;
    if ((rc = h2d(ws.predIdx, idx.data(), nms * sizeof(unsigned), fn, "the predecessors")) != NOVA_SUCCESS) return rc;
    dense_beliefs_kernel<<<r, 256>>>(n, r, rz, ws.Z, ws.B, ws.BT);
    if ((rc = check_launch(fn, "dense beliefs")) != NOVA_SUCCESS) return rc;
    ws.md = ExpModel{n, ns, m, z, r, rz, p->gamma, ws.S, ws.T, ws.O, ws.R, ws.Z, ws.B, ws.predStart, ws.predIdx,
                     ws.BT};
    ws.smem = 4 * (size_t)n * sizeof(float);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            ws.smem + 4096 > (size_t)optin) {
        cudaGetLastError();
        NOVA_ERR(fn, "Too many states for the expansion's shared-memory buffers.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (ws.smem > 40 * 1024) {
        cudaFuncSetAttribute(distinct_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws.smem);
        cudaFuncSetAttribute(random_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws.smem);
        cudaFuncSetAttribute(pema_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws.smem);
        cudaFuncSetAttribute(update_one_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws.smem);
    }
    return NOVA_SUCCESS;
}

bool valid_model(const POMDP *p) {
    return p != nullptr && p->n != 0 && p->ns != 0 && p->m != 0 && p->z != 0 && p->r != 0 && p->rz != 0 &&
           p->S != nullptr && p->T != nullptr && p->O != nullptr && p->R != nullptr && p->Z != nullptr &&
           p->B != nullptr;
}

// Lay out the random trajectories from the rand() stream and run them.
// fromB0: the _gpu form (every trajectory starts at belief 0, Bnew[0] is
// belief 0, no Pr(o) > 0 requirement). Returns Bnew [total][n] on the host.
int run_random(const POMDP *p, unsigned total, bool fromB0, std::vector<float> &Bnew, const char *fn) {
    ExpWorkspace ws;
    int rc = build_workspace(p, ws, fn);
    if (rc != NOVA_SUCCESS) return rc;
    seed_rand();
    std::vector<unsigned> start, first;
    std::vector<Step> steps;
    unsigned i = fromB0 ? 1u : 0u;
    while (i < total) {
        // A draw equal to RAND_MAX gives r (or m below); the reference would
        // read past its arrays there, this clamps to the last index.
        const unsigned b0 = fromB0 ? 0u : std::min(draw((float)p->r), p->r - 1);
        const unsigned h = draw((float)(p->horizon + 1));
        start.push_back(b0);
        first.push_back((unsigned)steps.size());
        for (unsigned t = 0; t < h; t++) {
            const unsigned a = draw((float)p->m);
            const float target = (float)rand() / (float)RAND_MAX;
            steps.push_back(Step{(unsigned)start.size() - 1, std::min(a, p->m - 1), target, i});
            i++;
            if (i >= total) break;
        }
    }
    first.push_back((unsigned)steps.size());
    // Trajectories without steps write nothing; drop them.
    std::vector<unsigned> s2, f2;
    for (size_t k = 0; k + 1 < first.size(); k++)
        if (first[k + 1] > first[k]) { s2.push_back(start[k]); f2.push_back(first[k]); }
    f2.push_back((unsigned)steps.size());
    float *dB = nullptr;
    unsigned *dStart = nullptr, *dFirst = nullptr;
    Step *dSteps = nullptr;
    const size_t n = p->n;
    struct Free {
        float *&b; unsigned *&s, *&f; Step *&st;
        ~Free() { cudaFree(b); cudaFree(s); cudaFree(f); cudaFree(st); }
    } guard{dB, dStart, dFirst, dSteps};
    if ((rc = dev_alloc(&dB, (size_t)total * n, fn, "the new beliefs")) != NOVA_SUCCESS) return rc;
    if (cudaMemset(dB, 0, (size_t)total * n * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to clear the new beliefs.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (!s2.empty()) {
        if ((rc = dev_alloc(&dStart, s2.size(), fn, "the trajectory starts")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dFirst, f2.size(), fn, "the trajectory offsets")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dSteps, steps.size(), fn, "the trajectory steps")) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(dStart, s2.data(), s2.size() * sizeof(unsigned), fn, "the trajectory starts")) != NOVA_SUCCESS)
            return rc;
        if ((rc = h2d(dFirst, f2.data(), f2.size() * sizeof(unsigned), fn, "the trajectory offsets")) != NOVA_SUCCESS)
            return rc;
        if ((rc = h2d(dSteps, steps.data(), steps.size() * sizeof(Step), fn, "the trajectory steps")) != NOVA_SUCCESS)
            return rc;
        random_kernel<<<(unsigned)s2.size(), kThreads, ws.smem>>>(ws.md, dStart, dFirst, dSteps, fromB0 ? 0 : 1, dB);
        if ((rc = check_launch(fn, "random trajectories")) != NOVA_SUCCESS) return rc;
    }
    if (fromB0) {
        // Bnew[0] = belief 0.
        std::vector<float> b0(n, 0.0f);
        for (unsigned j = 0; j < p->rz; j++) {
            const int s = p->Z[j];
            if (s < 0) break;
            b0[s] = p->B[j];
        }
        if ((rc = h2d(dB, b0.data(), n * sizeof(float), fn, "the initial belief")) != NOVA_SUCCESS) return rc;
    }
    Bnew.assign((size_t)total * n, 0.0f);
    return d2h(Bnew.data(), dB, (size_t)total * n * sizeof(float), fn, "the new beliefs");
}

}  // namespace
}  // namespace nova_gb300

using namespace nova_gb300;

extern "C" int pomdp_expand_random_cpu(POMDP *pomdp, unsigned int numBeliefsToAdd) {
    static const char *fn = "pomdp_expand_random_cpu";
    if (!valid_model(pomdp) || pomdp->horizon < 1 || numBeliefsToAdd == 0) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    std::vector<float> Bnew;
    int rc = run_random(pomdp, numBeliefsToAdd, false, Bnew, fn);
    if (rc != NOVA_SUCCESS) return rc;
    return pomdp_add_new_raw_beliefs_cpu(pomdp, numBeliefsToAdd, Bnew.data());
}

extern "C" int pomdp_expand_random_gpu(const POMDP *pomdp, unsigned int numThreads,
                                       unsigned int numDesiredBeliefPoints, unsigned int &maxNonZeroValues,
                                       float *&Bnew) {
    static const char *fn = "pomdp_expand_random_gpu";
    if (!valid_model(pomdp) || pomdp->horizon < 1 || numDesiredBeliefPoints <= 1 || Bnew != nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    (void)numThreads;  // launch shapes are fixed by the kernels
    std::vector<float> B;
    int rc = run_random(pomdp, numDesiredBeliefPoints, true, B, fn);
    if (rc != NOVA_SUCCESS) return rc;
    const size_t n = pomdp->n;
    unsigned maxNZ = 0;
    for (unsigned i = 1; i < numDesiredBeliefPoints; i++) {
        unsigned nz = 0;
        for (size_t s = 0; s < n; s++) nz += B[(size_t)i * n + s] > 0.0f ? 1u : 0u;
        maxNZ = std::max(maxNZ, nz);
    }
    maxNonZeroValues = maxNZ;
    Bnew = new float[(size_t)numDesiredBeliefPoints * n];
    memcpy(Bnew, B.data(), (size_t)numDesiredBeliefPoints * n * sizeof(float));
    return NOVA_SUCCESS;
}

extern "C" int pomdp_expand_distinct_beliefs_cpu(POMDP *pomdp) {
    static const char *fn = "pomdp_expand_distinct_beliefs_cpu";
    if (!valid_model(pomdp)) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    std::vector<float> Bnew;
    {
        ExpWorkspace ws;
        int rc = build_workspace(pomdp, ws, fn);
        if (rc != NOVA_SUCCESS) return rc;
        float *dB = nullptr;
        const size_t rn = (size_t)pomdp->r * pomdp->n;
        if ((rc = dev_alloc(&dB, rn, fn, "the new beliefs")) != NOVA_SUCCESS) return rc;
        distinct_kernel<<<pomdp->r, kThreads, ws.smem>>>(ws.md, dB);
        rc = check_launch(fn, "distinct beliefs");
        if (rc == NOVA_SUCCESS) {
            Bnew.assign(rn, 0.0f);
            rc = d2h(Bnew.data(), dB, rn * sizeof(float), fn, "the new beliefs");
        }
        cudaFree(dB);
        if (rc != NOVA_SUCCESS) return rc;
    }
    return pomdp_add_new_raw_beliefs_cpu(pomdp, pomdp->r, Bnew.data());
}

extern "C" int pomdp_expand_pema_cpu(POMDP *pomdp, const POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_expand_pema_cpu";
    if (!valid_model(pomdp) || policy == nullptr || policy->Gamma == nullptr || policy->r == 0 ||
            policy->n != pomdp->n) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned r = pomdp->r, n = pomdp->n;
    std::vector<float> Bnew(n, 0.0f);
    {
        ExpWorkspace ws;
        int rc = build_workspace(pomdp, ws, fn);
        if (rc != NOVA_SUCCESS) return rc;
        float *dGamma = nullptr, *dVal = nullptr, *dOut = nullptr;
        unsigned *dA = nullptr, *dO = nullptr;
        struct Free {
            float *&g, *&v, *&o; unsigned *&a, *&b;
            ~Free() { cudaFree(g); cudaFree(v); cudaFree(o); cudaFree(a); cudaFree(b); }
        } guard{dGamma, dVal, dOut, dA, dO};
        if ((rc = dev_alloc(&dGamma, (size_t)policy->r * n, fn, "the policy")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dVal, r, fn, "the error bounds")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dA, r, fn, "the best actions")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dO, r, fn, "the best observations")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&dOut, n, fn, "the new belief")) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(dGamma, policy->Gamma, (size_t)policy->r * n * sizeof(float), fn, "the policy")) !=
                NOVA_SUCCESS)
            return rc;
        pema_kernel<<<r, kThreads, ws.smem>>>(ws.md, policy->r, dGamma, dVal, dA, dO);
        if ((rc = check_launch(fn, "error bounds")) != NOVA_SUCCESS) return rc;
        std::vector<float> val(r);
        std::vector<unsigned> A(r), O(r);
        if ((rc = d2h(val.data(), dVal, r * sizeof(float), fn, "the error bounds")) != NOVA_SUCCESS) return rc;
        if ((rc = d2h(A.data(), dA, r * sizeof(unsigned), fn, "the best actions")) != NOVA_SUCCESS) return rc;
        if ((rc = d2h(O.data(), dO, r * sizeof(unsigned), fn, "the best observations")) != NOVA_SUCCESS) return rc;
        // The reference keeps the belief of the last strict increase of the
        // running maximum, i.e. the first belief attaining the maximum.
        float bStar = NOVA_FLT_MIN;
        unsigned win = kNoIndex;
        for (unsigned i = 0; i < r; i++)
            if (val[i] > bStar) { bStar = val[i]; win = i; }
        if (win != kNoIndex) {
            update_one_kernel<<<1, kThreads, ws.smem>>>(ws.md, win, A[win], O[win], dOut);
            if ((rc = check_launch(fn, "new belief")) != NOVA_SUCCESS) return rc;
            if ((rc = d2h(Bnew.data(), dOut, n * sizeof(float), fn, "the new belief")) != NOVA_SUCCESS) return rc;
        }
    }
    return pomdp_add_new_raw_beliefs_cpu(pomdp, 1, Bnew.data());
}

extern "C" int nova_gb300_expand_seed(unsigned int fixed, unsigned int seed) {
    g_seed.store(seed);
    g_seed_fixed.store(fixed ? 1u : 0u);
    return NOVA_SUCCESS;
}

// ---------------------------------------------------------------------------
// Sigma approximation (pomdp_sigma_cpu.cpp:49-118)
// ---------------------------------------------------------------------------

namespace nova_gb300 {
namespace {

// One thread per belief: sort its rz (value, state) entries by value,
// descending (equal values keep their support order), keep the top k,
// normalise them by their sum (added largest first) and report that sum.
__global__ void sigma_kernel(unsigned r, unsigned rz, unsigned k, const int *__restrict__ Z,
                             const float *__restrict__ B, int *__restrict__ Znew, float *__restrict__ Bnew,
                             float *__restrict__ sigmaB, float *__restrict__ scratchV, int *__restrict__ scratchS) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r) return;
    float *v = scratchV + (size_t)i * rz;
    int *st = scratchS + (size_t)i * rz;
    for (unsigned q = 0; q < rz; q++) {
        // Insertion sort keeps equal values in support order.
        const float x = B[(size_t)i * rz + q];
        const int y = Z[(size_t)i * rz + q];
        unsigned p = q;
        while (p > 0 && v[p - 1] < x) { v[p] = v[p - 1]; st[p] = st[p - 1]; p--; }
        v[p] = x;
        st[p] = y;
    }
    float sb = 0.0f;
    for (unsigned q = 0; q < k && q < rz; q++) sb = fadd(sb, v[q]);
    sigmaB[i] = sb;
    for (unsigned q = 0; q < k; q++) {
        const bool keep = q < rz && v[q] > 0.0f;
        Bnew[(size_t)i * k + q] = keep ? __fdiv_rn(v[q], sb) : 0.0f;
        Znew[(size_t)i * k + q] = keep ? st[q] : -1;
    }
}

}  // namespace
}  // namespace nova_gb300

extern "C" int pomdp_sigma_cpu(POMDP *pomdp, unsigned int numDesiredNonZeroValues, float &sigma) {
    static const char *fn = "pomdp_sigma_cpu";
    if (pomdp == nullptr || pomdp->z == 0 || pomdp->r == 0 || pomdp->rz == 0 || pomdp->Z == nullptr ||
            pomdp->B == nullptr || numDesiredNonZeroValues == 0) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned r = pomdp->r, rz = pomdp->rz, k = numDesiredNonZeroValues;
    int *dZ = nullptr, *dZn = nullptr, *dS = nullptr;
    float *dB = nullptr, *dBn = nullptr, *dSig = nullptr, *dV = nullptr;
    struct Free {
        int *&a, *&b, *&c; float *&d, *&e, *&f, *&g;
        ~Free() { cudaFree(a); cudaFree(b); cudaFree(c); cudaFree(d); cudaFree(e); cudaFree(f); cudaFree(g); }
    } guard{dZ, dZn, dS, dB, dBn, dSig, dV};
    int rc;
    const size_t rrz = (size_t)r * rz, rk = (size_t)r * k;
    if ((rc = dev_alloc(&dZ, rrz, fn, "the belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dB, rrz, fn, "the belief values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dS, rrz, fn, "the sorted states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dV, rrz, fn, "the sorted values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dZn, rk, fn, "the new belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dBn, rk, fn, "the new belief values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dSig, r, fn, "the belief sums")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(dZ, pomdp->Z, rrz * sizeof(int), fn, "the belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(dB, pomdp->B, rrz * sizeof(float), fn, "the belief values")) != NOVA_SUCCESS) return rc;
    sigma_kernel<<<ceil_div(r, 128), 128>>>(r, rz, k, dZ, dB, dZn, dBn, dSig, dV, dS);
    if ((rc = check_launch(fn, "sigma approximation")) != NOVA_SUCCESS) return rc;
    int *Znew = new int[rk];
    float *Bnew = new float[rk];
    std::vector<float> sig(r);
    if ((rc = d2h(Znew, dZn, rk * sizeof(int), fn, "the new belief states")) != NOVA_SUCCESS ||
            (rc = d2h(Bnew, dBn, rk * sizeof(float), fn, "the new belief values")) != NOVA_SUCCESS ||
            (rc = d2h(sig.data(), dSig, r * sizeof(float), fn, "the belief sums")) != NOVA_SUCCESS) {
        delete[] Znew;
        delete[] Bnew;
        return rc;
    }
    // sigma = min(1, min_i sigma_b), in belief order (pomdp_sigma_cpu.cpp:80-92).
    float s = 1.0f;
    for (unsigned i = 0; i < r; i++)
        if (sig[i] < s) s = sig[i];
    sigma = s;
    delete[] pomdp->Z;
    delete[] pomdp->B;
    pomdp->rz = k;
    pomdp->Z = Znew;
    pomdp->B = Bnew;
    return NOVA_SUCCESS;
}
