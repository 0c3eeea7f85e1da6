// nova-gb300: the point-based backup on the GB300, exact-order path, and
// the PBVI entry points (device buffers: pomdp_pbvi_*_gpu; host buffers:
// pomdp_pbvi_*_cpu).
//
// What one backup computes (pomdp_pbvi_cpu.cpp:37-162): for every belief i
// and action a,
//     j*(i,a,o) = argmax_j  sum_k B[i,k] * gamma * sum_l O(a,S,o) T(s_k,a,l) Gamma_j(S)
//     alpha_a   = R(.,a) + sum_o gamma * sum_l O T Gamma_{j*}(S)
//     a*(i)     = argmax_a  alpha_a . b_i ;   Gamma'_i = alpha_{a*},  pi_i = a*
// with the reference's sentinels (-1e10) and strict '>' (lowest index wins).
//
// Kernels (all FP32 with every product and sum rounded separately, in the
// reference's order, so results are bit-identical to the CPU path):
//   * tables_*          step-invariant successor lengths and coefficients
//                       C = fl(O(a,S,o) * T(s,a,l)) in two layouts
//   * dedup_*           bitwise-identical alpha rows collapse to the lowest
//                       index (they score identically, and lowest j wins)
//   * exact_score       per (i,a): all observations x all unique alphas, lanes
//                       over alphas reading the transposed alpha table
//                       (coalesced), coefficients broadcast from shared memory
//   * action_value      per (i,a): alpha_a on the belief support and its value
//   * assemble          per belief: action argmax, full alpha_{a*} over n states
// The tensor-core scoring (pbvi_tc.cu) replaces exact_score for rows whose
// argmax it can prove and hands the rest back to exact_score.

#include "pbvi.h"

#include <mutex>

#include <vector>
#include <algorithm>

#include <nova/constants.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_cpu.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_gpu.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

using nova::POMDP;
using nova::POMDPPBVICPU;
using nova::POMDPPBVIGPU;
using nova::POMDPAlphaVectors;
using nova::NovaPBVIStats;

namespace nova_gb300 {

constexpr unsigned kNone = 0xffffffffu;

// ---------------------------------------------------------------------------
// Step-invariant tables
// ---------------------------------------------------------------------------

__global__ void tables_len_kernel(unsigned rows, unsigned width, const int *__restrict__ idx,
                                  unsigned *__restrict__ len) {
    const unsigned row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    unsigned L = width;
    for (unsigned l = 0; l < width; l++) {
        if (idx[(size_t)row * width + l] < 0) { L = l; break; }
    }
    len[row] = L;
}

// C1[a][s][l][o] and C3[a][o][s][l] = fl(O(a,S(s,a,l),o) * T(s,a,l)), 0 past the row end.
__global__ void tables_coef_kernel(DevModel md, const unsigned *__restrict__ succLen, float *__restrict__ C1,
                                   float *__restrict__ C3) {
    const size_t total = (size_t)md.m * md.n * md.ns * md.z;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const unsigned o = (unsigned)(e % md.z);
        size_t t = e / md.z;
        const unsigned l = (unsigned)(t % md.ns);
        t /= md.ns;
        const unsigned s = (unsigned)(t % md.n);
        const unsigned a = (unsigned)(t / md.n);
        float c = 0.0f;
        if (l < succLen[(size_t)s * md.m + a]) {
            const size_t row = ((size_t)s * md.m + a) * md.ns + l;
            const int sp = md.S[row];
            c = fmul(md.O[((size_t)a * md.n + sp) * md.z + o], md.T[row]);
        }
        C1[e] = c;
        C3[(((size_t)a * md.z + o) * md.n + s) * md.ns + l] = c;
    }
}

// ---------------------------------------------------------------------------
// Dedup of alpha rows
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27; x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

__global__ void dedup_hash_kernel(const float *__restrict__ G, unsigned n, unsigned long long *__restrict__ hash) {
    const unsigned j = blockIdx.x;
    const unsigned *row = reinterpret_cast<const unsigned *>(G + (size_t)j * n);
    unsigned long long h = 0;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x)
        h += mix64(((unsigned long long)row[s] << 20) ^ (0x9e3779b97f4a7c15ull * (s + 1)));
    __shared__ unsigned long long red[32];
    for (int off = 16; off > 0; off >>= 1) h += __shfl_xor_sync(0xffffffffu, h, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = h;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (unsigned w = 0; w < (blockDim.x + 31) / 32; w++) t += red[w];
        hash[j] = t;
    }
}

__device__ bool rows_equal(const float *G, unsigned n, unsigned j1, unsigned j2) {
    const unsigned *a = reinterpret_cast<const unsigned *>(G + (size_t)j1 * n);
    const unsigned *b = reinterpret_cast<const unsigned *>(G + (size_t)j2 * n);
    for (unsigned s = 0; s < n; s++)
        if (a[s] != b[s]) return false;
    return true;
}

__global__ void dedup_rep_kernel(const unsigned long long *__restrict__ hash, const float *__restrict__ G,
                                 unsigned n, unsigned rows, unsigned *__restrict__ rep) {
    __shared__ unsigned long long tile[256];
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned long long myh = j < rows ? hash[j] : 0ull;
    unsigned r = j;
    bool found = false;
    const unsigned last = min(rows, (blockIdx.x + 1) * blockDim.x);  // no candidate beyond this block
    for (unsigned t0 = 0; t0 < last; t0 += 256) {
        __syncthreads();
        if (t0 + threadIdx.x < rows) tile[threadIdx.x] = hash[t0 + threadIdx.x];
        __syncthreads();
        if (j < rows && !found) {
            const unsigned lim = min(256u, j > t0 ? j - t0 : 0u);
            for (unsigned q = 0; q < lim; q++) {
                if (tile[q] == myh && rows_equal(G, n, t0 + q, j)) { r = t0 + q; found = true; break; }
            }
        }
    }
    if (j < rows) rep[j] = r;
}

// Single-block stream compaction of the rows that are their own representative.
__global__ void __launch_bounds__(1024) dedup_compact_kernel(const unsigned *__restrict__ rep, unsigned rows,
                                                             unsigned *__restrict__ uniqJ, unsigned *__restrict__ nU) {
    __shared__ unsigned warpSums[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (unsigned base = 0; base < rows; base += blockDim.x) {
        const unsigned j = base + threadIdx.x;
        const unsigned flag = (j < rows && rep[j] == j) ? 1u : 0u;
        // inclusive warp scan
        unsigned v = flag;
        const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= (unsigned)off) v += y;
        }
        if (lane == 31) warpSums[warp] = v;
        __syncthreads();
        if (warp == 0) {
            unsigned w = lane < (blockDim.x >> 5) ? warpSums[lane] : 0u;
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= (unsigned)off) w += y;
            }
            warpSums[lane] = w;  // inclusive
        }
        __syncthreads();
        const unsigned before = carry + (warp > 0 ? warpSums[warp - 1] : 0u) + v - flag;
        if (flag) uniqJ[before] = j;
        __syncthreads();
        if (threadIdx.x == 0) carry += warpSums[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *nU = carry;
}

// Gt[s][u] = G[uniqJ[u]][s]
__global__ void gather_transpose_kernel(const float *__restrict__ G, unsigned n, const unsigned *__restrict__ uniqJ,
                                        unsigned nU, float *__restrict__ Gt, size_t gtCols) {
    __shared__ float tile[32][33];
    const unsigned u0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
    for (unsigned k = threadIdx.y; k < 32; k += blockDim.y) {
        const unsigned u = u0 + k, s = s0 + threadIdx.x;
        tile[k][threadIdx.x] = (u < nU && s < n) ? G[(size_t)uniqJ[u] * n + s] : 0.0f;
    }
    __syncthreads();
    for (unsigned k = threadIdx.y; k < 32; k += blockDim.y) {
        const unsigned s = s0 + k, u = u0 + threadIdx.x;
        if (s < n && u < gtCols) Gt[(size_t)s * gtCols + u] = tile[threadIdx.x][k];
    }
}

// ---------------------------------------------------------------------------
// Exact scoring: value(i,a,o,u) in the order of pomdp_pbvi_cpu.cpp:50-83
// ---------------------------------------------------------------------------

// Better-than for the argmax: strictly larger value, or equal value and
// lower index. NaN is never better (the reference's `value > bestValue`).
__device__ __forceinline__ bool better(float v1, unsigned u1, float v2, unsigned u2) {
    return v1 > v2 || (v1 == v2 && u1 < u2);
}

template <int ZC>
__global__ void __launch_bounds__(128) exact_score_kernel(DevModel md, const unsigned *__restrict__ succLen,
        const unsigned *__restrict__ suppLen, const float *__restrict__ C1, const float *__restrict__ Gt,
        size_t gtCols, unsigned nU, const unsigned *__restrict__ items, unsigned nItems, unsigned splits,
        unsigned splitLen, float *__restrict__ partV, unsigned *__restrict__ partU) {
    extern __shared__ float smem[];
    float *Cs = smem;                                           // [ns][ZC]
    int *Ss = reinterpret_cast<int *>(Cs + (size_t)md.ns * ZC); // [ns]
    __shared__ float redV[4][ZC];
    __shared__ unsigned redU[4][ZC];
    __shared__ float runV[ZC];
    __shared__ unsigned runU[ZC];

    const unsigned tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned split = blockIdx.y;
    const unsigned uBegin = split * splitLen;
    const unsigned uEnd = min(nU, uBegin + splitLen);
    const float gamma = md.gamma;

    for (unsigned w = blockIdx.x; w < nItems; w += gridDim.x) {
        const unsigned ia = items[w];
        const unsigned i = ia / md.m, a = ia % md.m;
        const unsigned Li = suppLen[i];
        for (unsigned o0 = 0; o0 < md.z; o0 += ZC) {
            if (tid < ZC) { runV[tid] = NOVA_FLT_MIN; runU[tid] = kNone; }
            for (unsigned u0 = uBegin; u0 < uEnd; u0 += blockDim.x) {
                const unsigned u = u0 + tid;
                const bool valid = u < uEnd;
                float score[ZC];
#pragma unroll
                for (int q = 0; q < ZC; q++) score[q] = 0.0f;
                for (unsigned k = 0; k < Li; k++) {
                    const int s = md.Z[(size_t)i * md.rz + k];
                    const float b = md.B[(size_t)i * md.rz + k];
                    const unsigned Ls = succLen[(size_t)s * md.m + a];
                    __syncthreads();
                    const float *crow = C1 + (((size_t)a * md.n + s) * md.ns) * md.z + o0;
                    for (unsigned e = tid; e < Ls * ZC; e += blockDim.x) {
                        const unsigned l = e / ZC, q = e % ZC;
                        Cs[e] = (o0 + q < md.z) ? crow[(size_t)l * md.z + q] : 0.0f;
                    }
                    for (unsigned e = tid; e < Ls; e += blockDim.x) Ss[e] = md.S[((size_t)s * md.m + a) * md.ns + e];
                    __syncthreads();
                    if (valid) {
                        float vt[ZC];
#pragma unroll
                        for (int q = 0; q < ZC; q++) vt[q] = 0.0f;
                        for (unsigned l = 0; l < Ls; l++) {
                            const float g = Gt[(size_t)Ss[l] * gtCols + u];
#pragma unroll
                            for (int q = 0; q < ZC; q++) vt[q] = fadd(vt[q], fmul(Cs[l * ZC + q], g));
                        }
#pragma unroll
                        for (int q = 0; q < ZC; q++) score[q] = fadd(score[q], fmul(fmul(vt[q], gamma), b));
                    }
                }
                // Block argmax per observation over this chunk of alphas.
#pragma unroll
                for (int q = 0; q < ZC; q++) {
                    float v = valid ? score[q] : NOVA_FLT_MIN;
                    unsigned uu = valid ? u : kNone;
                    if (!(v > NOVA_FLT_MIN)) { v = NOVA_FLT_MIN; uu = kNone; }
                    for (int off = 16; off > 0; off >>= 1) {
                        const float v2 = __shfl_xor_sync(0xffffffffu, v, off);
                        const unsigned u2 = __shfl_xor_sync(0xffffffffu, uu, off);
                        if (better(v2, u2, v, uu)) { v = v2; uu = u2; }
                    }
                    if (lane == 0) { redV[warp][q] = v; redU[warp][q] = uu; }
                }
                __syncthreads();
                if (tid < ZC) {
                    float v = runV[tid];
                    unsigned uu = runU[tid];
                    for (unsigned ww = 0; ww < blockDim.x / 32; ww++)
                        if (redU[ww][tid] != kNone && better(redV[ww][tid], redU[ww][tid], v, uu)) {
                            v = redV[ww][tid]; uu = redU[ww][tid];
                        }
                    runV[tid] = v; runU[tid] = uu;
                }
                __syncthreads();
            }
            if (tid < ZC && o0 + tid < md.z) {
                const size_t p = ((size_t)w * md.z + o0 + tid) * splits + split;
                partV[p] = runV[tid];
                partU[p] = runU[tid];
            }
            __syncthreads();
        }
    }
}

// Merge split partials in alpha order; map unique index -> original j.
// When no alpha beats the -1e10 sentinel the reference keeps the previous
// observation's choice (bestj outlives the o loop, pomdp_pbvi_cpu.cpp:43-45);
// for the first observation it is undefined there and 0 here.
__global__ void exact_finalize_kernel(DevModel md, const unsigned *__restrict__ items, unsigned nItems,
                                      unsigned splits, const float *__restrict__ partV,
                                      const unsigned *__restrict__ partU, const unsigned *__restrict__ uniqJ,
                                      unsigned *__restrict__ jstar) {
    const unsigned w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nItems) return;
    const unsigned ia = items[w];
    unsigned prev = 0;
    for (unsigned o = 0; o < md.z; o++) {
        float v = NOVA_FLT_MIN;
        unsigned uu = kNone;
        for (unsigned sp = 0; sp < splits; sp++) {
            const size_t p = ((size_t)w * md.z + o) * splits + sp;
            if (partU[p] != kNone && better(partV[p], partU[p], v, uu)) { v = partV[p]; uu = partU[p]; }
        }
        const unsigned j = uu == kNone ? prev : uniqJ[uu];
        jstar[(size_t)ia * md.z + o] = j;
        prev = j;
    }
}

// ---------------------------------------------------------------------------
// Action values and assembly (pomdp_pbvi_cpu.cpp:88-101 and :128-157)
// ---------------------------------------------------------------------------

// gamma * sum_l C3 * G_j(S) for state s under action a, observation o, in the
// reference order (products left to right, sums sequential).
__device__ __forceinline__ float projected(const DevModel &md, const float *__restrict__ C3,
                                           const unsigned *__restrict__ succLen, const float *__restrict__ Gj,
                                           unsigned a, unsigned o, unsigned s) {
    const unsigned Ls = succLen[(size_t)s * md.m + a];
    const float *c = C3 + (((size_t)a * md.z + o) * md.n + s) * md.ns;
    const int *sp = md.S + ((size_t)s * md.m + a) * md.ns;
    float vt = 0.0f;
    for (unsigned l = 0; l < Ls; l++) vt = fadd(vt, fmul(c[l], Gj[sp[l]]));
    return fmul(vt, md.gamma);
}

// The same term with state s's successors already in registers (ss, Ls of
// them, at most kRegNs) and its coefficients read as float4 (ns a multiple
// of 4, rows 16-byte aligned): same operations in the same order.
constexpr unsigned kRegNs = 32;
__device__ __forceinline__ bool reg_form(const DevModel &md) { return md.ns <= kRegNs && md.ns % 4u == 0u; }
__device__ __forceinline__ float projected_regs(const DevModel &md, const float *__restrict__ C3,
                                                const int (&ss)[kRegNs], unsigned Ls, const float *__restrict__ Gj,
                                                unsigned a, unsigned o, unsigned s) {
    const float4 *c4 = reinterpret_cast<const float4 *>(C3 + (((size_t)a * md.z + o) * md.n + s) * md.ns);
    float g[kRegNs], c[kRegNs];
#pragma unroll
    for (unsigned q = 0; q < kRegNs / 4; q++) {
        if (4u * q < Ls) {
            const float4 v = __ldg(c4 + q);
            c[4 * q] = v.x; c[4 * q + 1] = v.y; c[4 * q + 2] = v.z; c[4 * q + 3] = v.w;
        }
    }
#pragma unroll
    for (unsigned l = 0; l < kRegNs; l++)
        if (l < Ls) g[l] = __ldg(Gj + ss[l]);
    float vt = 0.0f;
#pragma unroll
    for (unsigned l = 0; l < kRegNs; l++)
        if (l < Ls) vt = fadd(vt, fmul(c[l], g[l]));
    return fmul(vt, md.gamma);
}

// State s's successors under action a into registers (the first Ls).
__device__ __forceinline__ unsigned load_succ(const DevModel &md, const unsigned *__restrict__ succLen, unsigned a,
                                              unsigned s, int (&ss)[kRegNs]) {
    const unsigned Ls = __ldg(succLen + (size_t)s * md.m + a);
    const int *sp = md.S + ((size_t)s * md.m + a) * md.ns;
#pragma unroll
    for (unsigned l = 0; l < kRegNs; l++) ss[l] = l < Ls ? __ldg(sp + l) : 0;
    return Ls;
}

// One warp per (belief, action) item: alpha_a on the belief support, then
// value = sum_k alpha_a(s_k) * b_k in support order. Lane k takes support
// state k0 + k; observations run in the outer loop, so the warp's gathers
// of one observation's chosen alpha stay within one row.
__global__ void __launch_bounds__(256) action_value_kernel(DevModel md, const unsigned *__restrict__ succLen,
                                    const unsigned *__restrict__ suppLen, const float *__restrict__ C3,
                                    const float *__restrict__ G, const unsigned *__restrict__ jstar,
                                    const unsigned *__restrict__ items, unsigned nItems,
                                    float *__restrict__ actVal) {
    const unsigned warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (warpGlobal >= nItems) return;
    const unsigned ia = items ? items[warpGlobal] : warpGlobal;
    const unsigned i = ia / md.m, a = ia % md.m;
    const unsigned Li = suppLen[i];
    const bool regs = reg_form(md);
    float value = 0.0f;
    for (unsigned k0 = 0; k0 < Li; k0 += 32) {
        const unsigned k = k0 + lane;
        const bool v = k < Li;
        const unsigned s = v ? (unsigned)md.Z[(size_t)i * md.rz + k] : 0u;
        float alpha = v ? md.R[(size_t)s * md.m + a] : 0.0f;
        if (regs) {
            int ss[kRegNs];
            const unsigned Ls = v ? load_succ(md, succLen, a, s, ss) : 0u;
            for (unsigned o = 0; o < md.z; o++) {
                const float *Gj = G + (size_t)jstar[(size_t)ia * md.z + o] * md.n;
                if (v) alpha = fadd(alpha, projected_regs(md, C3, ss, Ls, Gj, a, o, s));
            }
        } else {
            for (unsigned o = 0; o < md.z; o++) {
                const float *Gj = G + (size_t)jstar[(size_t)ia * md.z + o] * md.n;
                if (v) alpha = fadd(alpha, projected(md, C3, succLen, Gj, a, o, s));
            }
        }
        const float p = v ? fmul(alpha, md.B[(size_t)i * md.rz + k]) : 0.0f;
        const unsigned cnt = min(32u, Li - k0);
        for (unsigned t = 0; t < cnt; t++) value = fadd(value, __shfl_sync(0xffffffffu, p, t));
    }
    if (lane == 0) actVal[ia] = value;
}

// One block per belief: action argmax (strict '>' from -1e10, lowest action
// on ties), then the full alpha of the best action over all n states. A
// belief whose every action fails to beat the sentinel keeps its old row
// and action, as in the reference.
__global__ void assemble_kernel(DevModel md, const unsigned *__restrict__ succLen, const float *__restrict__ C3,
                                const float *__restrict__ G, const unsigned *__restrict__ jstar,
                                const float *__restrict__ actVal, unsigned beliefBegin, float *__restrict__ dst,
                                unsigned *__restrict__ pi, float *__restrict__ rowOut, unsigned *__restrict__ actionOut) {
    const unsigned i = beliefBegin + blockIdx.x;
    __shared__ unsigned bestA;
    extern __shared__ unsigned jsh[];  // [z]
    if (threadIdx.x == 0) {
        float best = NOVA_FLT_MIN;
        unsigned ba = kNone;
        for (unsigned a = 0; a < md.m; a++) {
            const float v = actVal[(size_t)i * md.m + a];
            if (v > best) { best = v; ba = a; }
        }
        bestA = ba;
        if (actionOut) *actionOut = ba;
    }
    __syncthreads();
    const unsigned a = bestA;
    if (a == kNone) return;
    if (pi && threadIdx.x == 0) pi[i] = a;
    float *out = rowOut ? rowOut : dst + (size_t)i * md.n;
    const unsigned *js = jstar + ((size_t)i * md.m + a) * md.z;
    for (unsigned o = threadIdx.x; o < md.z; o += blockDim.x) jsh[o] = js[o];
    __syncthreads();
    if (reg_form(md)) {
        // The state's successors stay in registers across the observations.
        for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
            int ss[kRegNs];
            const unsigned Ls = load_succ(md, succLen, a, s, ss);
            float alpha = md.R[(size_t)s * md.m + a];
            for (unsigned o = 0; o < md.z; o++)
                alpha = fadd(alpha, projected_regs(md, C3, ss, Ls, G + (size_t)jsh[o] * md.n, a, o, s));
            out[s] = alpha;
        }
        return;
    }
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        float alpha = md.R[(size_t)s * md.m + a];
        for (unsigned o = 0; o < md.z; o++)
            alpha = fadd(alpha, projected(md, C3, succLen, G + (size_t)jsh[o] * md.n, a, o, s));
        out[s] = alpha;
    }
}

__global__ void iota_items_kernel(unsigned *items, unsigned count, unsigned first) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) items[t] = first + t;
}

// ---------------------------------------------------------------------------
// V(b) in FP64 (pomdp_alpha_vectors.cpp:52-79 reduced in double)
// ---------------------------------------------------------------------------

__global__ void row_dot_fp64_kernel(const float *__restrict__ G, unsigned n, const float *__restrict__ b,
                                    double *__restrict__ out) {
    const unsigned j = blockIdx.x;
    double acc = 0.0;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) acc += (double)G[(size_t)j * n + s] * (double)b[s];
    __shared__ double red[32];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned w = 0; w < (blockDim.x + 31) / 32; w++) t += red[w];
        out[j] = t;
    }
}

__global__ void argmax_fp64_kernel(const double *__restrict__ v, unsigned rows, const unsigned *__restrict__ pi,
                                   double *__restrict__ outV, unsigned *__restrict__ outA) {
    double best = (double)NOVA_FLT_MIN;
    unsigned bi = kNone;
    for (unsigned j = threadIdx.x; j < rows; j += blockDim.x)
        if (v[j] > best || (v[j] == best && bi != kNone && j < bi)) { best = v[j]; bi = j; }
    __shared__ double sv[256];
    __shared__ unsigned si[256];
    sv[threadIdx.x] = best; si[threadIdx.x] = bi;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned t = 1; t < blockDim.x; t++) {
            if (si[t] == kNone) continue;
            if (si[0] == kNone || sv[t] > sv[0] || (sv[t] == sv[0] && si[t] < si[0])) { sv[0] = sv[t]; si[0] = si[t]; }
        }
        *outV = sv[0];
        *outA = si[0] == kNone ? 0u : pi[si[0]];
    }
}

// ---------------------------------------------------------------------------
// Projection table: Proj[a][o][s][u] = gamma * sum_l fl(O(a,S,o) T(s,a,l)) * alpha_u(S)
// ---------------------------------------------------------------------------



// The reference recomputes this value (its Vtk after `Vtk *= gamma`,
// pomdp_pbvi_cpu.cpp:66-74 and :89-98) for every belief that has s in its
// support; it depends only on (a, o, s, alpha), so it is computed once per
// update here, with the same operands in the same order (bit-identical).
// One block per (a, s); threads over alphas read the transposed alpha table
// coalesced, the coefficients of the row are broadcast from shared memory,
// and each observation's values are written as one coalesced row segment.
template <int ZC>
__global__ void __launch_bounds__(256) proj_kernel(DevModel md, const unsigned *__restrict__ succLen,
                                                   const float *__restrict__ C1, const float *__restrict__ Gt,
                                                   size_t gtCols, unsigned nU, float *__restrict__ Proj,
                                                   size_t uCols, float one) {
    extern __shared__ float smem[];
    const unsigned long long one2 = pack_f32x2(one, one);
    float *Cs = smem;                                           // [ns][ZC]
    int *Ss = reinterpret_cast<int *>(Cs + (size_t)md.ns * ZC); // [ns]
    const unsigned a = blockIdx.x / md.n, s = blockIdx.x % md.n;
    const unsigned L = succLen[(size_t)s * md.m + a];
    const float gamma = md.gamma;
    for (unsigned e = threadIdx.x; e < L; e += blockDim.x) Ss[e] = md.S[((size_t)s * md.m + a) * md.ns + e];
    for (unsigned o0 = 0; o0 < md.z; o0 += ZC) {
        __syncthreads();
        const float *crow = C1 + (((size_t)a * md.n + s) * md.ns) * md.z + o0;
        for (unsigned e = threadIdx.x; e < L * ZC; e += blockDim.x) {
            const unsigned l = e / ZC, q = e % ZC;
            Cs[e] = (o0 + q < md.z) ? crow[(size_t)l * md.z + q] : 0.0f;
        }
        __syncthreads();
        const unsigned zc = min((unsigned)ZC, md.z - o0);
        float *out = Proj + (((size_t)a * md.z + o0) * md.n + s) * uCols;
        const size_t oStride = (size_t)md.n * uCols;
        // Two alphas per thread (u and u + blockDim) share every coefficient read.
        for (unsigned u0 = 0; u0 < nU; u0 += 2 * blockDim.x) {
            const unsigned ua = u0 + threadIdx.x, ub = ua + blockDim.x;
            const bool va = ua < nU, vb = ub < nU;
            // Observation pairs (q, q+1) per instruction, with the exact
            // f32x2 form of fadd(acc, fmul(c, g)) described at
            // common.h (fma of the product by a run-time 1.0).
            unsigned long long acc0[ZC / 2], acc1[ZC / 2];
#pragma unroll
            for (int q = 0; q < ZC / 2; q++) { acc0[q] = 0ull; acc1[q] = 0ull; }
            for (unsigned l = 0; l < L; l++) {
                const float *grow = Gt + (size_t)Ss[l] * gtCols;
                const float g0 = va ? grow[ua] : 0.0f;
                const float g1 = vb ? grow[ub] : 0.0f;
                const unsigned long long gg0 = pack_f32x2(g0, g0), gg1 = pack_f32x2(g1, g1);
                const ulonglong2 *c2 = reinterpret_cast<const ulonglong2 *>(Cs + l * ZC);
#pragma unroll
                for (int q4 = 0; q4 < ZC / 4; q4++) {
                    const ulonglong2 c = c2[q4];
                    acc0[2 * q4 + 0] = fma_f32x2(mul_f32x2(c.x, gg0), one2, acc0[2 * q4 + 0]);
                    acc1[2 * q4 + 0] = fma_f32x2(mul_f32x2(c.x, gg1), one2, acc1[2 * q4 + 0]);
                    acc0[2 * q4 + 1] = fma_f32x2(mul_f32x2(c.y, gg0), one2, acc0[2 * q4 + 1]);
                    acc1[2 * q4 + 1] = fma_f32x2(mul_f32x2(c.y, gg1), one2, acc1[2 * q4 + 1]);
                }
            }
#pragma unroll
            for (int q = 0; q < ZC; q++) {
                if ((unsigned)q < zc) {
                    if (va) out[(size_t)q * oStride + ua] = fmul(f32x2_part(acc0[q / 2], q & 1), gamma);
                    if (vb) out[(size_t)q * oStride + ub] = fmul(f32x2_part(acc1[q / 2], q & 1), gamma);
                }
            }
        }
    }
}

// The state-contiguous layout [m][z][uRows][sCols] (see proj_state_lanes_kernel).
constexpr unsigned kProjTileS = 8;
constexpr unsigned kStateMajorMinStates = 1024;
constexpr int kProjUPL = 2;  // alphas per lane of the state-contiguous projection

// State-contiguous table, register form: one block per (a, 8 consecutive
// states) and column range of the alphas; lane (sl, ul) of every warp owns
// state s0 + sl and UPL alphas (the block's 8 warps cover 32*UPL alphas per
// step). Each lane reads its state's coefficients from shared memory
// (per-state blocks padded by 4 floats, so the 8 states of a warp fall in
// distinct banks) and keeps 32 observations' sums in registers; for every
// (o, alpha) the 8 lanes of one alpha write the 8 states' values as one
// 32-byte sector, straight from registers. Successor lists are staged
// successor-major ([l][8 states]), so the 8 states' l-th successors sit in
// 8 banks, and each lane's transposed-alpha gathers run two successors
// ahead of the arithmetic.
template <int ZC, int UPL>
__global__ void __launch_bounds__(256, UPL == 1 ? 3 : 2) proj_state_lanes_kernel(
        DevModel md, const unsigned *__restrict__ succLen, const float *__restrict__ C1,
        const float *__restrict__ Gt, size_t gtCols, unsigned nU, float *__restrict__ Proj, size_t uRows,
        size_t sCols, unsigned uRange, float one) {
    extern __shared__ float smem[];
    const unsigned cStride = md.ns * ZC + 4;
    float *Cs = smem;                                                   // [8][cStride]
    int *Ss = reinterpret_cast<int *>(Cs + (size_t)kProjTileS * cStride);  // [ns][8]
    __shared__ unsigned Ls[kProjTileS];
    const unsigned long long one2 = pack_f32x2(one, one);
    const unsigned tilesS = (md.n + kProjTileS - 1) / kProjTileS;
    const unsigned a = blockIdx.x / tilesS, s0 = (blockIdx.x % tilesS) * kProjTileS;
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned sl = lane >> 2, ul = lane & 3;
    const unsigned s = s0 + sl;
    const bool live = s < md.n;
    const float gamma = md.gamma;
    if (threadIdx.x < kProjTileS)
        Ls[threadIdx.x] = s0 + threadIdx.x < md.n ? succLen[(size_t)(s0 + threadIdx.x) * md.m + a] : 0u;
    for (unsigned e = threadIdx.x; e < kProjTileS * md.ns; e += blockDim.x) {
        const unsigned st = e / md.ns, l = e % md.ns;
        Ss[l * kProjTileS + st] = s0 + st < md.n ? md.S[((size_t)(s0 + st) * md.m + a) * md.ns + l] : 0;
    }
    for (unsigned o0 = 0; o0 < md.z; o0 += ZC) {
        __syncthreads();
        for (unsigned e = threadIdx.x; e < kProjTileS * md.ns * ZC; e += blockDim.x) {
            const unsigned st = e / (md.ns * ZC), rem = e % (md.ns * ZC), l = rem / ZC, q = rem % ZC;
            Cs[st * cStride + rem] = (s0 + st < md.n && l < Ls[st] && o0 + q < md.z)
                ? C1[(((size_t)a * md.n + s0 + st) * md.ns + l) * md.z + o0 + q] : 0.0f;
        }
        __syncthreads();
        const unsigned zc = min((unsigned)ZC, md.z - o0);
        const unsigned L = Ls[sl];
        const float *cw = Cs + (size_t)sl * cStride;
        const int *sw = Ss + sl;
        const unsigned uBegin = blockIdx.y * uRange, uEnd = min(nU, uBegin + uRange);
        for (unsigned u0 = uBegin + warp * 4u * UPL; u0 < uEnd; u0 += 32u * UPL) {
            unsigned uu[UPL];
            bool v[UPL];
#pragma unroll
            for (int j = 0; j < UPL; j++) {
                uu[j] = u0 + ul + 4u * j;
                v[j] = live && uu[j] < uEnd;
            }
            unsigned long long acc[UPL][ZC / 2];
#pragma unroll
            for (int j = 0; j < UPL; j++)
#pragma unroll
                for (int q = 0; q < ZC / 2; q++) acc[j][q] = 0ull;
            float gn[UPL], gn2[UPL];
            if (L > 0) {
                const float *grow = Gt + (size_t)sw[0] * gtCols;
                const float *grow2 = Gt + (size_t)sw[(L > 1 ? 1 : 0) * kProjTileS] * gtCols;
#pragma unroll
                for (int j = 0; j < UPL; j++) {
                    gn[j] = v[j] ? grow[uu[j]] : 0.0f;
                    gn2[j] = v[j] ? grow2[uu[j]] : 0.0f;
                }
            }
            for (unsigned l = 0; l < L; l++) {
                unsigned long long gg[UPL];
#pragma unroll
                for (int j = 0; j < UPL; j++) gg[j] = pack_f32x2(gn[j], gn[j]);
                const float *grow = Gt + (size_t)sw[(l + 2 < L ? l + 2 : L - 1) * kProjTileS] * gtCols;
#pragma unroll
                for (int j = 0; j < UPL; j++) {
                    gn[j] = gn2[j];
                    gn2[j] = v[j] ? grow[uu[j]] : 0.0f;
                }
                const ulonglong2 *c2 = reinterpret_cast<const ulonglong2 *>(cw + l * ZC);
#pragma unroll
                for (int q4 = 0; q4 < ZC / 4; q4++) {
                    const ulonglong2 c = c2[q4];
#pragma unroll
                    for (int j = 0; j < UPL; j++) {
                        acc[j][2 * q4 + 0] = fma_f32x2(mul_f32x2(c.x, gg[j]), one2, acc[j][2 * q4 + 0]);
                        acc[j][2 * q4 + 1] = fma_f32x2(mul_f32x2(c.y, gg[j]), one2, acc[j][2 * q4 + 1]);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < ZC; q++) {
                if ((unsigned)q < zc) {
#pragma unroll
                    for (int j = 0; j < UPL; j++)
                        if (v[j])
                            Proj[(((size_t)a * md.z + o0 + q) * uRows + uu[j]) * sCols + s] =
                                fmul(f32x2_part(acc[j][q / 2], q & 1), gamma);
                }
            }
        }
    }
}

// Exact scan of whole (a*z+o, belief) rows over the unique alphas using the
// projection table: value(u) = sum_k fl(Proj[ao][s_k][u] * B[i,k]) in
// support order (pomdp_pbvi_cpu.cpp:50-83), argmax with the lowest index on
// ties and the -1e10 sentinel. One block per row. The alphas are scanned in
// column chunks [u0, u1) so that the (a, o) slice being read stays in L2
// while the rows of that (a, o) (consecutive in the list) use it; a chunk
// after the first merges with the running best of the earlier ones, which
// hold lower indices (so ties keep the earlier alpha).
__global__ void __launch_bounds__(256) scan_rows_kernel(DevModel md, const unsigned *__restrict__ suppLen,
                                                        const ProjView pv, unsigned u0,
                                                        unsigned u1, const unsigned *__restrict__ rowList,
                                                        unsigned nRows, const unsigned *__restrict__ nRowsDev,
                                                        float *__restrict__ runV,
                                                        unsigned *__restrict__ runU, int first) {
    extern __shared__ float sh[];
    float *bk = sh;                                              // [rz]
    unsigned *sk = reinterpret_cast<unsigned *>(sh + md.rz);     // [rz]
    __shared__ float redV[8];
    __shared__ unsigned redU[8];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (nRowsDev) nRows = min(nRows, *nRowsDev);
    for (unsigned w = blockIdx.x; w < nRows; w += gridDim.x) {
        const unsigned row = rowList ? rowList[w] : w;
        const unsigned ao = row / md.r, i = row % md.r;
        const unsigned Li = suppLen[i];
        __syncthreads();
        for (unsigned k = threadIdx.x; k < Li; k += blockDim.x) {
            bk[k] = md.B[(size_t)i * md.rz + k];
            sk[k] = (unsigned)md.Z[(size_t)i * md.rz + k];
        }
        __syncthreads();
        const float *P = pv.slab(ao);
        float best = NOVA_FLT_MIN;
        unsigned bu = kNone;
        for (unsigned u = u0 + threadIdx.x; u < u1; u += blockDim.x) {
            float v = 0.0f;
            for (unsigned k = 0; k < Li; k++) v = fadd(v, fmul(__ldg(P + pv.at(sk[k], u)), bk[k]));
            if (v > best) { best = v; bu = u; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const float v2 = __shfl_xor_sync(0xffffffffu, best, off);
            const unsigned u2 = __shfl_xor_sync(0xffffffffu, bu, off);
            if (u2 != kNone && (bu == kNone || better(v2, u2, best, bu))) { best = v2; bu = u2; }
        }
        if (lane == 0) { redV[warp] = best; redU[warp] = bu; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (unsigned ww = 1; ww < blockDim.x / 32; ww++)
                if (redU[ww] != kNone && (bu == kNone || better(redV[ww], redU[ww], best, bu))) {
                    best = redV[ww]; bu = redU[ww];
                }
            if (!first) {
                const unsigned pu = runU[w];
                if (pu != kNone && (bu == kNone || !(best > runV[w]))) { best = runV[w]; bu = pu; }
            }
            runV[w] = best;
            runU[w] = bu;
        }
    }
}

// Final choice of each scanned row (kNone where nothing beat the sentinel).
__global__ void scan_finish_kernel(DevModel md, const unsigned *__restrict__ rowList, unsigned nRows,
                                   const unsigned *__restrict__ nRowsDev,
                                   const unsigned *__restrict__ runU, const unsigned *__restrict__ uniqJ,
                                   unsigned *__restrict__ ustar, unsigned *__restrict__ jstar) {
    const unsigned w = blockIdx.x * blockDim.x + threadIdx.x;
    if (nRowsDev) nRows = min(nRows, *nRowsDev);
    if (w >= nRows) return;
    const unsigned row = rowList ? rowList[w] : w;
    const unsigned ao = row / md.r, i = row % md.r;
    const size_t js = ((size_t)i * md.m + ao / md.z) * md.z + ao % md.z;
    const unsigned bu = runU[w];
    ustar[js] = bu;
    jstar[js] = bu == kNone ? kNone : uniqJ[bu];
}

// Rows with no alpha above the -1e10 sentinel take the previous
// observation's choice (0 for the first), as the reference's bestj does.
__global__ void sentinel_fixup_kernel(DevModel md, const unsigned *__restrict__ uniqJ, unsigned *__restrict__ ustar,
                                      unsigned *__restrict__ jstar) {
    const unsigned ia = blockIdx.x * blockDim.x + threadIdx.x;
    if (ia >= md.r * md.m) return;
    unsigned prevU = 0, prevJ = 0;
    for (unsigned o = 0; o < md.z; o++) {
        const size_t js = (size_t)ia * md.z + o;
        if (jstar[js] == kNone) {
            // uniqJ[0] == 0: the first row is always its own representative
            jstar[js] = prevJ;
            ustar[js] = prevU;
        }
        prevJ = jstar[js];
        prevU = ustar[js];
    }
}

// Action values from the projection table (one warp per (belief, action)):
// alpha_a(s_k) = R(s_k,a) + sum_o Proj[a][o][s_k][u*], value = sum_k alpha * b_k.
__global__ void action_value_proj_kernel(DevModel md, const unsigned *__restrict__ suppLen,
                                         const ProjView pv,
                                         const unsigned *__restrict__ ustar, float *__restrict__ actVal) {
    const unsigned warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (warpGlobal >= md.r * md.m) return;
    const unsigned ia = warpGlobal;
    const unsigned i = ia / md.m, a = ia % md.m;
    const unsigned Li = suppLen[i];
    float value = 0.0f;
    for (unsigned k0 = 0; k0 < Li; k0 += 32) {
        const unsigned k = k0 + lane;
        float p = 0.0f;
        if (k < Li) {
            const int s = md.Z[(size_t)i * md.rz + k];
            float alpha = md.R[(size_t)s * md.m + a];
            for (unsigned o = 0; o < md.z; o++) {
                const unsigned u = ustar[(size_t)ia * md.z + o];
                alpha = fadd(alpha, pv.slab(a * md.z + o)[pv.at(s, u)]);
            }
            p = fmul(alpha, md.B[(size_t)i * md.rz + k]);
        }
        const unsigned cnt = min(32u, Li - k0);
        for (unsigned t = 0; t < cnt; t++) value = fadd(value, __shfl_sync(0xffffffffu, p, t));
    }
    if (lane == 0) actVal[ia] = value;
}

// Assembly from the projection table: Gamma'_i(s) = R(s,a*) + sum_o
// Proj[a*][o][s][u*_o], the reference's alpha for the best action
// (pomdp_pbvi_cpu.cpp:128-145, 88-101) with its additions in observation
// order. One block per belief; each thread issues a chunk of independent
// loads before the sequential additions.
__global__ void __launch_bounds__(256) assemble_proj_kernel(DevModel md, const ProjView pv,
                                                            const unsigned *__restrict__ ustar,
                                                            const float *__restrict__ actVal, float *__restrict__ dst,
                                                            unsigned *__restrict__ pi) {
    const unsigned i = blockIdx.x;
    __shared__ unsigned bestA;
    extern __shared__ unsigned ush[];  // [z]
    if (threadIdx.x == 0) {
        float best = NOVA_FLT_MIN;
        unsigned ba = kNone;
        for (unsigned a = 0; a < md.m; a++) {
            const float v = actVal[(size_t)i * md.m + a];
            if (v > best) { best = v; ba = a; }
        }
        bestA = ba;
    }
    __syncthreads();
    const unsigned a = bestA;
    if (a == kNone) return;
    if (threadIdx.x == 0) pi[i] = a;
    const unsigned *us = ustar + ((size_t)i * md.m + a) * md.z;
    for (unsigned o = threadIdx.x; o < md.z; o += blockDim.x) ush[o] = us[o];
    __syncthreads();
    const float *P = pv.slab(a * md.z);
    const size_t oStride = pv.slice;
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        float alpha = md.R[(size_t)s * md.m + a];
        const float *Ps = P + s * pv.sStride;
        unsigned o = 0;
        for (; o + 8 <= md.z; o += 8) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; q++) v[q] = __ldg(Ps + (size_t)(o + q) * oStride + ush[o + q] * pv.uStride);
#pragma unroll
            for (int q = 0; q < 8; q++) alpha = fadd(alpha, v[q]);
        }
        for (; o < md.z; o++) alpha = fadd(alpha, __ldg(Ps + (size_t)o * oStride + ush[o] * pv.uStride));
        dst[(size_t)i * md.n + s] = alpha;
    }
}

// ---------------------------------------------------------------------------
// BackupEngine
// ---------------------------------------------------------------------------

BackupEngine::~BackupEngine() {
    cudaDeviceSynchronize();
    for (auto &g : graph)
        if (g) cudaGraphExecDestroy(g);
    if (tc) tc_release(tc);
    cudaFree(succLen); cudaFree(suppLen); cudaFree(C1); cudaFree(C3);
    cudaFree(hash); cudaFree(rep); cudaFree(uniqJ); cudaFree(nUniqueDev); cudaFree(Gt);
    cudaFree(jstar); cudaFree(actVal); cudaFree(partV); cudaFree(partU); cudaFree(items); cudaFree(itemCount);
    cudaFree(keptCount);
    cudaFree(dotScratch); cudaFree(bDense); cudaFree(resultA); cudaFree(resultV); cudaFree(rowScratch);
    cudaFree(vnb); cudaFree(vnp1b); cudaFree(btilde);
    cudaFree(Proj); cudaFree(ustar); cudaFree(scanV); cudaFree(scanU);
    if (eventsMade)
        for (auto &e : ev) cudaEventDestroy(e);
}

int BackupEngine::build(const DevModel &model, const char *fn) {
    md = model;
    int rc;
    // Work queued by earlier synchronous copies must be complete before the
    // tables read the model.
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;
    const size_t nm = (size_t)md.n * md.m;
    const size_t coef = nm * md.ns * md.z;
    if ((rc = dev_alloc(&succLen, nm, fn, "the successor lengths")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&suppLen, md.r, fn, "the belief support lengths")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&C1, coef, fn, "the projection coefficients")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&C3, coef, fn, "the projection coefficients (successor-major)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&hash, md.r, fn, "the alpha hashes")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&rep, md.r, fn, "the alpha representatives")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&uniqJ, md.r, fn, "the unique alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&nUniqueDev, 1, fn, "the unique alpha count")) != NOVA_SUCCESS) return rc;
    gtCols = round_up(md.r, 32);
    if ((rc = dev_alloc(&Gt, (size_t)md.n * gtCols, fn, "the transposed alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&jstar, (size_t)md.r * md.m * md.z, fn, "the chosen alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ustar, (size_t)md.r * md.m * md.z, fn, "the chosen unique alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&actVal, (size_t)md.r * md.m, fn, "the action values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&items, (size_t)md.r * md.m, fn, "the work list")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&itemCount, 1, fn, "the work list count")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&keptCount, 1, fn, "the kept-belief count")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dotScratch, md.r, fn, "the FP64 values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bDense, md.n, fn, "the belief")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&resultA, 1, fn, "the action")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&resultV, 1, fn, "the value")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&rowScratch, md.n, fn, "the alpha row")) != NOVA_SUCCESS) return rc;
    if (!eventsMade) {
        for (auto &e : ev) cudaEventCreate(&e);
        eventsMade = true;
    }
    tables_len_kernel<<<ceil_div(nm, 256), 256>>>((unsigned)nm, md.ns, md.S, succLen);
    if ((rc = check_launch(fn, "successor lengths")) != NOVA_SUCCESS) return rc;
    tables_len_kernel<<<ceil_div(md.r, 256), 256>>>(md.r, md.rz, md.Z, suppLen);
    if ((rc = check_launch(fn, "support lengths")) != NOVA_SUCCESS) return rc;
    tables_coef_kernel<<<std::min<size_t>(ceil_div(coef, 256), 65535u * 8u), 256>>>(md, succLen, C1, C3);
    if ((rc = check_launch(fn, "projection coefficients")) != NOVA_SUCCESS) return rc;
    return sync_device(fn);
}

int BackupEngine::dedup(const float *src, unsigned rows, unsigned *nUnique, const char *fn) {
    int rc;
    if (rows == 0) { *nUnique = 0; return NOVA_SUCCESS; }
    dedup_hash_kernel<<<rows, 128, 0, stream>>>(src, md.n, hash);
    if ((rc = check_launch(fn, "alpha hash")) != NOVA_SUCCESS) return rc;
    dedup_rep_kernel<<<ceil_div(rows, 256), 256, 0, stream>>>(hash, src, md.n, rows, rep);
    if ((rc = check_launch(fn, "alpha dedup")) != NOVA_SUCCESS) return rc;
    dedup_compact_kernel<<<1, 1024, 0, stream>>>(rep, rows, uniqJ, nUniqueDev);
    if ((rc = check_launch(fn, "alpha compaction")) != NOVA_SUCCESS) return rc;
    unsigned h = 0;
    if (cudaMemcpyAsync(&h, nUniqueDev, sizeof(unsigned), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to read the number of unique alpha-vectors.");
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    *nUnique = h;
    // Transposed unique alphas for the exact scan.
    dim3 grid(ceil_div(std::max(h, 1u), 32), ceil_div(md.n, 32));
    gather_transpose_kernel<<<grid, dim3(32, 8), 0, stream>>>(src, md.n, uniqJ, h, Gt, gtCols);
    return check_launch(fn, "alpha transpose");
}

template <int ZC>
static void launch_exact(BackupEngine &e, const unsigned *items, unsigned nItems, unsigned nU, unsigned splits,
                         unsigned splitLen, unsigned grid) {
    const size_t smem = (size_t)e.md.ns * ZC * sizeof(float) + (size_t)e.md.ns * sizeof(int);
    if (smem > 48 * 1024) cudaFuncSetAttribute(exact_score_kernel<ZC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    exact_score_kernel<ZC><<<dim3(grid, splits), 128, smem, e.stream>>>(e.md, e.succLen, e.suppLen, e.C1, e.Gt,
            e.gtCols, nU, items, nItems, splits, splitLen, e.partV, e.partU);
}

int BackupEngine::exact_score(const unsigned *itemList, unsigned nItems, unsigned nU, const char *fn) {
    if (nItems == 0) return NOVA_SUCCESS;
    int rc;
    // Split the alpha range so that the grid covers the device.
    const unsigned target = 152u * 8u;
    unsigned splits = 1;
    if (nItems < target) splits = std::min(ceil_div(target, nItems), std::max(1u, ceil_div(nU, 128)));
    splits = std::max(1u, std::min(splits, 1024u));
    const unsigned splitLen = (unsigned)round_up(ceil_div(std::max(nU, 1u), splits), 128);
    splits = std::max(1u, ceil_div(std::max(nU, 1u), splitLen));
    const size_t need = (size_t)nItems * md.z * splits;
    if (need > partCap) {
        cudaFree(partV); cudaFree(partU);
        partV = nullptr; partU = nullptr; partCap = 0;
        if ((rc = dev_alloc(&partV, need, fn, "the partial maxima")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&partU, need, fn, "the partial arg-maxima")) != NOVA_SUCCESS) return rc;
        partCap = need;
    }
    const unsigned grid = std::min(nItems, 65535u);
    const size_t smem32 = (size_t)md.ns * 32 * sizeof(float) + md.ns * sizeof(int);
    if (md.z >= 16 && smem32 <= 200 * 1024) launch_exact<32>(*this, itemList, nItems, nU, splits, splitLen, grid);
    else if (md.z >= 4 && (size_t)md.ns * 8 * 4 <= 200 * 1024) launch_exact<8>(*this, itemList, nItems, nU, splits, splitLen, grid);
    else if ((size_t)md.ns * 2 * 4 <= 200 * 1024) launch_exact<2>(*this, itemList, nItems, nU, splits, splitLen, grid);
    else {
        NOVA_ERR(fn, "Too many successors per state for the exact scoring kernel.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if ((rc = check_launch(fn, "exact belief scoring")) != NOVA_SUCCESS) return rc;
    exact_finalize_kernel<<<ceil_div(nItems, 128), 128, 0, stream>>>(md, itemList, nItems, splits, partV, partU,
                                                                      uniqJ, jstar);
    return check_launch(fn, "exact belief scoring (merge)");
}

bool BackupEngine::ensure_proj(unsigned nU) {
    if (projUnavailable || tableNever) return false;
    const size_t cols = round_up(std::max(nU, 1u), 32);
    const size_t sCols = round_up(md.n, kProjTileS);
    projSCols = sCols;
    const size_t need = (size_t)md.m * md.z * sCols * cols;
    if (need <= projCap) {
        projCols = cols;
        return true;
    }
    // Capacity for the largest possible alpha set in either layout, allocated once.
    const size_t full = (size_t)md.m * md.z * sCols * round_up(md.r, 32);
    size_t freeB = 0, totalB = 0;
    cudaMemGetInfo(&freeB, &totalB);
    cudaFree(Proj);
    Proj = nullptr;
    projCap = 0;
    if (full * sizeof(float) + (1ull << 30) > freeB || cudaMalloc(&Proj, full * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        Proj = nullptr;
        projUnavailable = true;
        return false;
    }
    projCap = full;
    projCols = cols;
    return true;
}

int BackupEngine::project(unsigned nU, const char *fn) {
    if (projStateMajor) {
        const unsigned zc = md.z >= 16 ? 32u : 8u;
        const size_t smem = (size_t)kProjTileS * (md.ns * zc + 4) * sizeof(float) +
                            (size_t)kProjTileS * md.ns * sizeof(int);
        if (!projAttrDone) {
            cudaFuncSetAttribute(proj_state_lanes_kernel<32, kProjUPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(proj_state_lanes_kernel<8, kProjUPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(proj_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            cudaFuncSetAttribute(proj_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
            projAttrDone = true;
        }
        // Column ranges of about 32 MB of the transposed alphas (multiples of 32*UPL).
        const unsigned uRange = (unsigned)std::max<size_t>(
            32 * kProjUPL, ((32ull << 20) / ((size_t)md.n * sizeof(float))) / (32 * kProjUPL) * (32 * kProjUPL));
        const dim3 blocks(md.m * ceil_div(md.n, kProjTileS), ceil_div(std::max(nU, 1u), uRange));
        if (zc == 32)
            proj_state_lanes_kernel<32, kProjUPL><<<blocks, 256, smem, stream>>>(md, succLen, C1, Gt, gtCols, nU, Proj,
                                                                             projCols, projSCols, uRange, 1.0f);
        else
            proj_state_lanes_kernel<8, kProjUPL><<<blocks, 256, smem, stream>>>(md, succLen, C1, Gt, gtCols, nU, Proj,
                                                                            projCols, projSCols, uRange, 1.0f);
        return check_launch(fn, "projection table");
    }
    const size_t smem32 = (size_t)md.ns * 32 * sizeof(float) + md.ns * sizeof(int);
    const unsigned blocks = md.m * md.n;
    if (!projAttrDone) {
        cudaFuncSetAttribute(proj_state_lanes_kernel<32, kProjUPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(proj_state_lanes_kernel<8, kProjUPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(proj_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(proj_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        projAttrDone = true;
    }
    if (md.z >= 16 && smem32 <= 200 * 1024) {
        proj_kernel<32><<<blocks, 256, smem32, stream>>>(md, succLen, C1, Gt, gtCols, nU, Proj, projCols, 1.0f);
    } else {
        const size_t smem8 = (size_t)md.ns * 8 * sizeof(float) + md.ns * sizeof(int);
        proj_kernel<8><<<blocks, 256, smem8, stream>>>(md, succLen, C1, Gt, gtCols, nU, Proj, projCols, 1.0f);
    }
    return check_launch(fn, "projection table");
}

int BackupEngine::scan_rows(const unsigned *rowList, unsigned nRows, unsigned nU, const char *fn,
                            const unsigned *nRowsDev) {
    if (nRows == 0) return NOVA_SUCCESS;
    int rc;
    if ((size_t)nRows > scanCap) {
        cudaFree(scanV); cudaFree(scanU);
        scanV = nullptr; scanU = nullptr; scanCap = 0;
        if ((rc = dev_alloc(&scanV, nRows, fn, "the scan maxima")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&scanU, nRows, fn, "the scan arg-maxima")) != NOVA_SUCCESS) return rc;
        scanCap = nRows;
    }
    // Column chunk: one (a, o) slice of at most ~48 MB stays L2-resident.
    size_t chunk = ((48ull << 20) / ((size_t)md.n * sizeof(float))) / 256 * 256;
    if (chunk < 256) chunk = 256;
    const unsigned grid = std::min(nRows, 152u * 16u);
    for (size_t u0 = 0; u0 < std::max(nU, 1u); u0 += chunk) {
        const unsigned u1 = (unsigned)std::min<size_t>(nU, u0 + chunk);
        scan_rows_kernel<<<grid, 256, 2 * md.rz * sizeof(float), stream>>>(md, suppLen, proj_view(), (unsigned)u0,
                                                                          u1, rowList, nRows, nRowsDev, scanV,
                                                                          scanU, u0 == 0 ? 1 : 0);
        if ((rc = check_launch(fn, "exact row scan")) != NOVA_SUCCESS) return rc;
    }
    scan_finish_kernel<<<ceil_div(nRows, 256), 256, 0, stream>>>(md, rowList, nRows, nRowsDev, scanU, uniqJ, ustar,
                                                                 jstar);
    if ((rc = check_launch(fn, "exact row scan (finish)")) != NOVA_SUCCESS) return rc;
    sentinel_fixup_kernel<<<ceil_div((size_t)md.r * md.m, 256), 256, 0, stream>>>(md, uniqJ, ustar, jstar);
    return check_launch(fn, "sentinel fixup");
}

int BackupEngine::scan_rows_direct(const unsigned *rowList, unsigned nRows, unsigned nU, const char *fn) {
    if (nRows == 0) return NOVA_SUCCESS;
    int rc;
    const size_t allItems = (size_t)md.r * md.m;
    if ((rc = tc_rows_to_items(*this, rowList, nRows, fn)) != NOVA_SUCCESS) return rc;
    unsigned nItems = 0;
    if (cudaMemcpyAsync(&nItems, itemCount, sizeof(unsigned), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to read the number of (belief, action) pairs to score.");
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    if (nItems > allItems) {
        NOVA_ERR(fn, "Inconsistent (belief, action) list.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    return exact_score(items, nItems, nU, fn);
}

int BackupEngine::fill_items(unsigned first, unsigned count, const char *fn) {
    if (count == 0) return NOVA_SUCCESS;
    iota_items_kernel<<<ceil_div(count, 256), 256, 0, stream>>>(items, count, first);
    return check_launch(fn, "work list");
}

int BackupEngine::assemble(const float *src, float *dst, unsigned *pi, int onlyBelief, float *dstRowOverride,
                           unsigned *actionOut, const char *fn) {
    int rc;
    const unsigned firstBelief = onlyBelief >= 0 ? (unsigned)onlyBelief : 0u;
    const unsigned nBeliefs = onlyBelief >= 0 ? 1u : md.r;
    const unsigned nItems = nBeliefs * md.m;
    const unsigned *itemList = nullptr;
    if (onlyBelief >= 0) {
        iota_items_kernel<<<ceil_div(nItems, 256), 256, 0, stream>>>(items, nItems, firstBelief * md.m);
        if ((rc = check_launch(fn, "work list")) != NOVA_SUCCESS) return rc;
        itemList = items;
    }
    if (useProjNow && onlyBelief < 0)
        action_value_proj_kernel<<<ceil_div((size_t)nItems * 32, 256), 256, 0, stream>>>(md, suppLen, proj_view(),
                                                                                         ustar, actVal);
    else
        action_value_kernel<<<ceil_div((size_t)nItems * 32, 256), 256, 0, stream>>>(md, succLen, suppLen, C3, src,
                                                                                    jstar, itemList, nItems, actVal);
    if ((rc = check_launch(fn, "action values")) != NOVA_SUCCESS) return rc;
    if (onlyBelief < 0 && !capturing) cudaEventRecord(ev[6], stream);
    if (useProjNow && onlyBelief < 0)
        assemble_proj_kernel<<<nBeliefs, 256, md.z * sizeof(unsigned), stream>>>(md, proj_view(), ustar, actVal,
                                                                                  dst, pi);
    else
        assemble_kernel<<<nBeliefs, 256, md.z * sizeof(unsigned), stream>>>(md, succLen, C3, src, jstar, actVal,
                                                                             firstBelief, dst, pi, dstRowOverride,
                                                                             actionOut);
    return check_launch(fn, "alpha assembly");
}

// Beliefs whose every action value fails to beat the sentinel: the assembly
// leaves their row and action untouched (pomdp_pbvi_cpu.cpp:128-145).
__global__ void count_kept_kernel(const float *__restrict__ actVal, unsigned r, unsigned m, unsigned *count) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r) return;
    for (unsigned a = 0; a < m; a++)
        if (actVal[(size_t)i * m + a] > NOVA_FLT_MIN) return;
    atomicAdd(count, 1u);
}

int BackupEngine::count_kept(unsigned *out, const char *fn) {
    if (cudaMemsetAsync(keptCount, 0, sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to clear the kept-belief count.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    count_kept_kernel<<<ceil_div(md.r, 256), 256, 0, stream>>>(actVal, md.r, md.m, keptCount);
    int rc = check_launch(fn, "kept beliefs");
    if (rc != NOVA_SUCCESS) return rc;
    if (cudaMemcpyAsync(out, keptCount, sizeof(unsigned), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to read the kept-belief count.");
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    return NOVA_SUCCESS;
}

int BackupEngine::backup_all(const float *src, unsigned rGamma, float *dst, unsigned *pi, const char *fn) {
    int rc;
    memset(&stats, 0, sizeof(stats));
    identityUniq = false;  // the dedup below rewrites uniqJ
    const unsigned long long launches0 = launch_count();
    cudaEventRecord(ev[0], stream);
    unsigned nU = 0;
    if ((rc = dedup(src, rGamma, &nU, fn)) != NOVA_SUCCESS) return rc;
    stats.uniqueAlphas = nU;
    cudaEventRecord(ev[1], stream);
    const unsigned allItems = md.r * md.m;
    // With room for the projection table every exact score is a 64-term
    // dot product over it: the plain form scans every row over it, and the
    // tensor-core form re-scores its near-ties and scans its unresolved rows
    // with it. Without it, the tensor-core form re-scores its near-ties from
    // the alphas directly and scores the (belief, action) pairs of its
    // unresolved rows in full, and the plain form scores every pair so.
    useProjNow = ensure_proj(nU);
    const bool wantTc = (scoring == NOVA_SCORING_BF16 || scoring == NOVA_SCORING_FP16) &&
                        tc_supported(md) && nU >= kTcMinUnique && !tcUnavailable;
    // Tensor-core updates of large models read the table by candidate and by
    // chosen alpha (assembly reads whole columns) and, in FP16, leave almost
    // no row to the exact scan, so they use the state-contiguous layout; the
    // exact scan reads whole rows and keeps the alpha-contiguous one, as do
    // smaller models and updates after one that left more than 1 % of its
    // rows to the scan (BF16's wider margin does).
    {
        const unsigned zc = md.z >= 16 ? 32u : 8u;
        const size_t smemSM = (size_t)kProjTileS * (md.ns * zc + 4) * sizeof(float) +
                              (size_t)kProjTileS * md.ns * sizeof(int);
        projStateMajor = wantTc && state_major_wanted(smemSM);
    }
    if (useProjNow && (rc = project(nU, fn)) != NOVA_SUCCESS) return rc;
    if (wantTc && tc == nullptr && tc_build(*this, fn) != NOVA_SUCCESS) tcUnavailable = true;
    cudaEventRecord(ev[2], stream);
    if (wantTc && tc != nullptr) {
        unsigned nRows = 0;
        const unsigned *rowList = nullptr;
        if ((rc = tc_score(*this, src, nU, &nRows, &rowList, fn)) != NOVA_SUCCESS) return rc;
        cudaEventRecord(ev[5], stream);
        stats.scoring = scoring;
        stats.rowsOverflow = nRows;
        lastScanFrac = (float)nRows / (float)((size_t)md.m * md.z * md.r);
        if (useProjNow) {
            if ((rc = scan_rows(rowList, nRows, nU, fn)) != NOVA_SUCCESS) return rc;
        } else if ((rc = scan_rows_direct(rowList, nRows, nU, fn)) != NOVA_SUCCESS) {
            return rc;
        }
    } else if (useProjNow) {
        cudaEventRecord(ev[5], stream);
        stats.scoring = NOVA_SCORING_EXACT;
        if ((rc = scan_rows(nullptr, md.r * md.m * md.z, nU, fn)) != NOVA_SUCCESS) return rc;
    } else {
        iota_items_kernel<<<ceil_div(allItems, 256), 256, 0, stream>>>(items, allItems, 0);
        if ((rc = check_launch(fn, "work list")) != NOVA_SUCCESS) return rc;
        cudaEventRecord(ev[5], stream);
        stats.scoring = NOVA_SCORING_EXACT;
        if ((rc = exact_score(items, allItems, nU, fn)) != NOVA_SUCCESS) return rc;
    }
    cudaEventRecord(ev[3], stream);
    if ((rc = assemble(src, dst, pi, -1, nullptr, nullptr, fn)) != NOVA_SUCCESS) return rc;
    cudaEventRecord(ev[4], stream);
    if (cudaEventSynchronize(ev[4]) != cudaSuccess) {
        cudaGetLastError();
        return sync_device(fn);
    }
    cudaEventElapsedTime(&stats.msDedup, ev[0], ev[1]);
    cudaEventElapsedTime(&stats.msProject, ev[1], ev[2]);
    cudaEventElapsedTime(&stats.msScore, ev[2], ev[5]);
    cudaEventElapsedTime(&stats.msRescore, ev[5], ev[3]);
    cudaEventElapsedTime(&stats.msActions, ev[3], ev[6]);
    cudaEventElapsedTime(&stats.msAssemble, ev[6], ev[4]);
    cudaEventElapsedTime(&stats.msTotal, ev[0], ev[4]);
    stats.launches = (unsigned)(launch_count() - launches0);
    if (stats.tcGroups != 0) tc_tune_feedback(*this, stats.msScore + stats.msRescore, nU);
    const unsigned derr = tc_device_error();
    if (derr != 0) {
        NOVA_ERR(fn, "A device-side wait timed out; results of this update are invalid.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    return NOVA_SUCCESS;
}

bool BackupEngine::state_major_wanted(size_t smemSM) const {
    return md.n > kStateMajorMinStates && smemSM <= 200 * 1024 &&
           (scoring == NOVA_SCORING_FP16 || scoring == NOVA_SCORING_BF16) && lastScanFrac <= 0.01f;
}

bool BackupEngine::fixed_ready() const {
    return tc != nullptr && !tcUnavailable && tc_schedule_fixed(*this) && Proj != nullptr && !projUnavailable &&
           projCap >= (size_t)md.m * md.z * std::max(projSCols, (size_t)md.n) * round_up(md.r, 32) &&
           scanCap >= (size_t)md.m * md.z * md.r && identityUniq &&
           (scoring == NOVA_SCORING_BF16 || scoring == NOVA_SCORING_FP16);
}

int BackupEngine::fixed_pre(const float *src, bool tensor, const char *fn) {
    int rc;
    const unsigned nU = md.r;
    dim3 grid(ceil_div(nU, 32), ceil_div(md.n, 32));
    gather_transpose_kernel<<<grid, dim3(32, 8), 0, stream>>>(src, md.n, uniqJ, nU, Gt, gtCols);
    if ((rc = check_launch(fn, "alpha transpose")) != NOVA_SUCCESS) return rc;
    useProjNow = ensure_proj(nU);
    if (!useProjNow) return NOVA_ERROR_KERNEL_EXECUTION;
    {
        const unsigned zc = md.z >= 16 ? 32u : 8u;
        const size_t smemSM = (size_t)kProjTileS * (md.ns * zc + 4) * sizeof(float) +
                              (size_t)kProjTileS * md.ns * sizeof(int);
        projStateMajor = tensor && state_major_wanted(smemSM);
    }
    if ((rc = project(nU, fn)) != NOVA_SUCCESS) return rc;
    return tensor ? tc_prepare(*this, src, nU, fn) : NOVA_SUCCESS;
}

int BackupEngine::fixed_post(const float *src, float *dst, unsigned *pi, bool tensor, const char *fn) {
    int rc;
    const unsigned nU = md.r;
    if (tensor) {
        if ((rc = tc_finish(*this, fn)) != NOVA_SUCCESS) return rc;
        rc = scan_rows(tc_row_list(*this), md.m * md.z * md.r, nU, fn, itemCount);
    } else {
        rc = scan_rows(nullptr, md.m * md.z * md.r, nU, fn);
    }
    if (rc != NOVA_SUCCESS) return rc;
    return assemble(src, dst, pi, -1, nullptr, nullptr, fn);
}

int BackupEngine::backup_fixed(const float *src, float *dst, unsigned *pi, const char *fn) {
    int rc;
    if ((rc = fixed_pre(src, true, fn)) != NOVA_SUCCESS) return rc;
    if ((rc = tc_gemm(*this, false, fn)) != NOVA_SUCCESS) return rc;
    return fixed_post(src, dst, pi, true, fn);
}

int BackupEngine::fixed_setup(const char *fn) {
    int rc;
    if (!identityUniq) {
        if ((rc = fill_items(0, md.r, fn)) != NOVA_SUCCESS) return rc;
        if (cudaMemcpyAsync(uniqJ, items, (size_t)md.r * sizeof(unsigned), cudaMemcpyDeviceToDevice, stream) !=
                cudaSuccess) {
            cudaGetLastError();
            return NOVA_ERROR_KERNEL_EXECUTION;
        }
        identityUniq = true;
    }
    const size_t rows = (size_t)md.m * md.z * md.r;
    if (scanCap < rows) {
        cudaFree(scanV); cudaFree(scanU);
        scanV = nullptr; scanU = nullptr; scanCap = 0;
        if ((rc = dev_alloc(&scanV, rows, fn, "the scan maxima")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&scanU, rows, fn, "the scan arg-maxima")) != NOVA_SUCCESS) return rc;
        scanCap = rows;
    }
    return NOVA_SUCCESS;
}

// Selections of the last backup: for belief i, the action a = pi[i] whose
// alpha became GammaPrime[i] and, per observation o, the alpha index j* that
// alpha took for (i, a, o). The projection-table path keeps its choices as
// unique-alpha indices (mapped back through uniqJ, the lowest original index
// of each distinct row, which is the reference's choice among equal rows).
__global__ void record_selection_kernel(unsigned r, unsigned m, unsigned z, const unsigned *__restrict__ pi,
                                        int fromUnique, const unsigned *__restrict__ ustar,
                                        const unsigned *__restrict__ uniqJ, const unsigned *__restrict__ jstar,
                                        unsigned *__restrict__ actOut, unsigned *__restrict__ selOut) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)r * z) return;
    const unsigned i = (unsigned)(idx / z), o = (unsigned)(idx % z);
    unsigned a = pi[i];
    if (a >= m) a = 0;
    const size_t k = ((size_t)i * m + a) * z + o;
    unsigned j;
    if (fromUnique) {
        const unsigned u = ustar[k];
        j = u == kNone ? 0u : uniqJ[u];
    } else {
        j = jstar[k];
        if (j == kNone) j = 0;
    }
    selOut[idx] = j;
    if (o == 0) actOut[i] = a;
}

int BackupEngine::record(const unsigned *pi, unsigned *actOut, unsigned *selOut, const char *fn) {
    record_selection_kernel<<<ceil_div((size_t)md.r * md.z, 256), 256, 0, stream>>>(
        md.r, md.m, md.z, pi, useProjNow ? 1 : 0, ustar, uniqJ, jstar, actOut, selOut);
    int rc = check_launch(fn, "selection record");
    if (rc != NOVA_SUCCESS) return rc;
    return sync_device(fn);
}

// ---------------------------------------------------------------------------
// Solver workspaces
// ---------------------------------------------------------------------------

struct PbviGpuWorkspace : Workspace {
    BackupEngine eng;
    bool built = false;
    const void *modelKey[6] = {};   // device model pointers the tables were built from
    float *d_Gamma = nullptr, *d_GammaPrime = nullptr;
    unsigned *d_pi = nullptr;
    ~PbviGpuWorkspace() override {
        cudaDeviceSynchronize();
        cudaFree(d_Gamma); cudaFree(d_GammaPrime); cudaFree(d_pi);
    }
};

struct PbviCpuWorkspace : Workspace {
    BackupEngine eng;
    bool built = false;
    int *S = nullptr; float *T = nullptr, *O = nullptr, *R = nullptr; int *Z = nullptr; float *B = nullptr;
    float *Gamma = nullptr, *GammaPrime = nullptr;
    unsigned *pi = nullptr;
    float *hostGamma = nullptr, *hostGammaPrime = nullptr;
    unsigned *hostPi = nullptr;
    bool hostPinned = false;  // the three host arrays are page-locked (cudaHostRegister)
    ~PbviCpuWorkspace() override {
        cudaDeviceSynchronize();
        if (hostPinned) {
            cudaHostUnregister(hostGamma);
            cudaHostUnregister(hostGammaPrime);
            cudaHostUnregister(hostPi);
            cudaGetLastError();
        }
        cudaFree(S); cudaFree(T); cudaFree(O); cudaFree(R); cudaFree(Z); cudaFree(B);
        cudaFree(Gamma); cudaFree(GammaPrime); cudaFree(pi);
    }
};

static DevModel device_model(const POMDP *p) {
    DevModel md;
    md.n = p->n; md.ns = p->ns; md.m = p->m; md.z = p->z; md.r = p->r; md.rz = p->rz; md.gamma = p->gamma;
    md.S = p->d_S; md.T = p->d_T; md.O = p->d_O; md.R = p->d_R; md.Z = p->d_Z; md.B = p->d_B;
    return md;
}

// Upload a host POMDP into device arrays owned by a workspace.
template <typename W>
static int upload_model(W *ws, const POMDP *p, DevModel *md, const char *fn) {
    const size_t nms = (size_t)p->n * p->m * p->ns, mnz = (size_t)p->m * p->n * p->z, nm = (size_t)p->n * p->m,
                 rrz = (size_t)p->r * p->rz;
    int rc;
    if ((rc = dev_alloc(&ws->S, nms, fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->T, nms, fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->O, mnz, fn, "the observation transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->R, nm, fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->Z, rrz, fn, "the non-zero belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->B, rrz, fn, "the belief points")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->S, p->S, nms * sizeof(int), fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->T, p->T, nms * sizeof(float), fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->O, p->O, mnz * sizeof(float), fn, "the observation transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->R, p->R, nm * sizeof(float), fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->Z, p->Z, rrz * sizeof(int), fn, "the non-zero belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->B, p->B, rrz * sizeof(float), fn, "the belief points")) != NOVA_SUCCESS) return rc;
    md->n = p->n; md->ns = p->ns; md->m = p->m; md->z = p->z; md->r = p->r; md->rz = p->rz; md->gamma = p->gamma;
    md->S = ws->S; md->T = ws->T; md->O = ws->O; md->R = ws->R; md->Z = ws->Z; md->B = ws->B;
    return NOVA_SUCCESS;
}

// Shared validation of pomdp_pbvi_cpu.cpp:192-200 / pomdp_pbvi_gpu.cu:266-274.
static bool pomdp_shape_invalid(const POMDP *p) {
    return p == nullptr || p->n == 0 || p->ns == 0 || p->m == 0 || p->z == 0 || p->r == 0 || p->rz == 0 ||
           p->gamma < 0.0f || p->gamma > 1.0f || p->horizon < 1;
}

}  // namespace nova_gb300

using namespace nova_gb300;

// ===========================================================================
// Device-buffer PBVI (pomdp_pbvi_gpu.cu)
// ===========================================================================

static PbviGpuWorkspace *pbvi_gpu_ws(const POMDPPBVIGPU *pbvi) {
    std::lock_guard<std::mutex> lock(registry_mutex());
    return find_workspace<PbviGpuWorkspace>(pbvi);
}

namespace nova_gb300 {
BackupEngine *pbvi_gpu_engine(const POMDPPBVIGPU *pbvi) {
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    return ws != nullptr && ws->built ? &ws->eng : nullptr;
}
}  // namespace nova_gb300

extern "C" int pomdp_pbvi_uninitialize_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi) {
    (void)pomdp;
    if (pbvi == nullptr) {
        NOVA_ERR("pomdp_pbvi_uninitialize_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pbvi->currentHorizon = 0;
    int result = NOVA_SUCCESS;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *ws = find_workspace<PbviGpuWorkspace>(pbvi);
        if (ws != nullptr) {
            if (pbvi->d_Gamma == ws->d_Gamma) pbvi->d_Gamma = nullptr;
            if (pbvi->d_GammaPrime == ws->d_GammaPrime) pbvi->d_GammaPrime = nullptr;
            if (pbvi->d_pi == ws->d_pi) pbvi->d_pi = nullptr;
            registry().erase(pbvi);
        }
    }
    // Fields this library did not allocate are freed as the reference does
    // (pomdp_pbvi_gpu.cu:312-358).
    float **fields[3] = {&pbvi->d_Gamma, &pbvi->d_GammaPrime, &pbvi->d_alphaBA};
    for (float **f : fields) {
        if (*f != nullptr && dev_free(*f, "pomdp_pbvi_uninitialize_gpu", "the alpha-vectors") != NOVA_SUCCESS)
            result = NOVA_ERROR_DEVICE_FREE;
        *f = nullptr;
    }
    if (pbvi->d_pi != nullptr && dev_free(pbvi->d_pi, "pomdp_pbvi_uninitialize_gpu", "pi") != NOVA_SUCCESS)
        result = NOVA_ERROR_DEVICE_FREE;
    pbvi->d_pi = nullptr;
    return result;
}

extern "C" int pomdp_pbvi_initialize_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi) {
    static const char *fn = "pomdp_pbvi_initialize_gpu";
    if (pomdp == nullptr || pbvi == nullptr || pomdp->n == 0 || pomdp->r == 0 || pbvi->GammaInitial == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pbvi->currentHorizon = 0;
    unsigned scoring = NOVA_SCORING_FP16;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *old = find_workspace<PbviGpuWorkspace>(pbvi);
        if (old != nullptr) {
            scoring = old->eng.scoring;
            if (pbvi->d_Gamma == old->d_Gamma) pbvi->d_Gamma = nullptr;
            if (pbvi->d_GammaPrime == old->d_GammaPrime) pbvi->d_GammaPrime = nullptr;
            if (pbvi->d_pi == old->d_pi) pbvi->d_pi = nullptr;
            registry().erase(pbvi);
        }
    }
    std::unique_ptr<PbviGpuWorkspace> ws(new PbviGpuWorkspace());
    ws->eng.scoring = scoring;
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    int rc;
    if ((rc = dev_alloc(&ws->d_Gamma, rn, fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->d_Gamma, pbvi->GammaInitial, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_GammaPrime, rn, fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->d_GammaPrime, pbvi->GammaInitial, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_pi, pomdp->r, fn, "pi")) != NOVA_SUCCESS) return rc;
    if (cudaMemset(ws->d_pi, 0, pomdp->r * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to clear pi.");
        return NOVA_ERROR_MEMCPY_TO_DEVICE;
    }
    pbvi->d_Gamma = ws->d_Gamma;
    pbvi->d_GammaPrime = ws->d_GammaPrime;
    pbvi->d_pi = ws->d_pi;
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[pbvi] = std::move(ws);
    return NOVA_SUCCESS;
}

// Tables are built on first use and rebuilt if the device model changed.
static int ensure_built(PbviGpuWorkspace *ws, const POMDP *pomdp, const char *fn) {
    const void *key[6] = {pomdp->d_S, pomdp->d_T, pomdp->d_O, pomdp->d_R, pomdp->d_Z, pomdp->d_B};
    if (ws->built && memcmp(key, ws->modelKey, sizeof(key)) == 0 && ws->eng.md.r == pomdp->r &&
            ws->eng.md.n == pomdp->n)
        return NOVA_SUCCESS;
    if (ws->built) {
        const unsigned scoring = ws->eng.scoring;
        ws->eng.~BackupEngine();
        new (&ws->eng) BackupEngine();
        ws->eng.scoring = scoring;
        ws->built = false;
    }
    int rc = ws->eng.build(device_model(pomdp), fn);
    if (rc != NOVA_SUCCESS) return rc;
    memcpy(ws->modelKey, key, sizeof(key));
    ws->built = true;
    return NOVA_SUCCESS;
}

// Graph mode: once the solver scores on the tensor cores with a fixed
// schedule, an update is the replay of a CUDA graph of backup_fixed (no host
// read-back inside), captured once per direction Gamma -> GammaPrime and
// GammaPrime -> Gamma on a private stream and launched on the solver's
// stream; the call still returns after the update is complete.
//
// A capture must not overlap a device-wide synchronisation or allocation
// in another host thread (the batched solve runs many solvers at once), so
// captures hold capture_lock() exclusively and every other update, and the
// batched solve's other calls, hold it shared.
std::shared_mutex &nova_gb300::capture_lock() {
    static std::shared_mutex m;
    return m;
}

static bool graph_wanted(const BackupEngine &e) {
    return e.graphMode && e.tc != nullptr && !e.tcUnavailable && tc_schedule_fixed(e) && e.Proj != nullptr &&
           !e.projUnavailable && (e.scoring == NOVA_SCORING_BF16 || e.scoring == NOVA_SCORING_FP16);
}

static int graph_dir(const BackupEngine &e, const float *src) {
    return src == e.graphSrc[0] ? 0 : src == e.graphSrc[1] ? 1 : (e.graph[0] == nullptr ? 0 : 1);
}

static bool graph_needs_capture(const BackupEngine &e, const float *src) {
    const int dir = graph_dir(e, src);
    return !e.identityUniq || e.graph[dir] == nullptr || e.graphSrc[dir] != src;
}

// Under capture_lock() held exclusively.
static int graph_prepare(BackupEngine &e, const float *src, float *dst, unsigned *pi, const char *fn) {
    int rc;
    if ((rc = e.fixed_setup(fn)) != NOVA_SUCCESS) return rc;
    if (!e.fixed_ready()) {
        e.graphMode = false;
        return NOVA_SUCCESS;
    }
    const int dir = graph_dir(e, src);
    if (e.graph[dir] != nullptr && e.graphSrc[dir] == src) return NOVA_SUCCESS;
    if (e.graph[dir]) { cudaGraphExecDestroy(e.graph[dir]); e.graph[dir] = nullptr; }
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        e.graphMode = false;  // stay with ordinary updates
        return NOVA_SUCCESS;
    }
    const cudaStream_t saved = e.stream;
    e.stream = cs;
    e.capturing = true;
    const unsigned long long l0 = launch_count();
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        rc = e.backup_fixed(src, dst, pi, fn);
        ok = cudaStreamEndCapture(cs, &g) == cudaSuccess && rc == NOVA_SUCCESS && g != nullptr;
    }
    const long long captured = (long long)(launch_count() - l0);
    add_launches(-captured);  // captured, not run
    e.stream = saved;
    e.capturing = false;
    cudaGraphExec_t exec = nullptr;
    if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (!ok) {
        cudaGetLastError();
        e.graphMode = false;  // ordinary updates from now on
        return NOVA_SUCCESS;
    }
    e.graph[dir] = exec;
    e.graphSrc[dir] = src;
    e.graphLaunches[dir] = (unsigned)captured;
    return NOVA_SUCCESS;
}

// Under capture_lock() held shared.
static int graph_replay(BackupEngine &e, const float *src, bool *done, const char *fn) {
    *done = false;
    if (!graph_wanted(e) || graph_needs_capture(e, src)) return NOVA_SUCCESS;
    const int dir = graph_dir(e, src);
    memset(&e.stats, 0, sizeof(e.stats));
    if (cudaGraphLaunch(e.graph[dir], e.stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to launch the update graph.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    add_launches(e.graphLaunches[dir]);
    if (cudaStreamSynchronize(e.stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "The update graph failed.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (tc_device_error() != 0) {
        NOVA_ERR(fn, "A device-side wait timed out; results of this update are invalid.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    e.stats.scoring = e.scoring;
    e.stats.uniqueAlphas = e.md.r;
    e.stats.launches = e.graphLaunches[dir];
    *done = true;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_update_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi) {
    static const char *fn = "pomdp_pbvi_update_gpu";
    if (pomdp_shape_invalid(pomdp) || pbvi == nullptr || pomdp->d_S == nullptr || pomdp->d_T == nullptr ||
            pomdp->d_O == nullptr || pomdp->d_R == nullptr || pomdp->d_Z == nullptr || pomdp->d_B == nullptr ||
            pbvi->d_Gamma == nullptr || pbvi->d_GammaPrime == nullptr || pbvi->d_pi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized (call pomdp_pbvi_initialize_gpu).");
        return NOVA_ERROR_INVALID_DATA;
    }
    std::shared_lock<std::shared_mutex> lock(nova_gb300::capture_lock());
    int rc = ensure_built(ws, pomdp, fn);
    if (rc != NOVA_SUCCESS) return rc;
    const bool even = (pbvi->currentHorizon % 2u) == 0u;
    const float *src = even ? pbvi->d_Gamma : pbvi->d_GammaPrime;
    float *dst = even ? pbvi->d_GammaPrime : pbvi->d_Gamma;
    BackupEngine &e = ws->eng;
    if (graph_wanted(e) && graph_needs_capture(e, src)) {
        lock.unlock();
        {
            std::unique_lock<std::shared_mutex> excl(nova_gb300::capture_lock());
            rc = graph_prepare(e, src, dst, pbvi->d_pi, fn);
        }
        lock.lock();
        if (rc != NOVA_SUCCESS) return rc;
    }
    bool byGraph = false;
    if ((rc = graph_replay(e, src, &byGraph, fn)) != NOVA_SUCCESS) return rc;
    if (!byGraph && (rc = e.backup_all(src, pomdp->r, dst, pbvi->d_pi, fn)) != NOVA_SUCCESS) return rc;
    pbvi->currentHorizon++;
    e.stats.horizon = pbvi->currentHorizon;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_update_record_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, unsigned int *d_action,
                                            unsigned int *d_select) {
    static const char *fn = "pomdp_pbvi_update_record_gpu";
    if (d_action == nullptr || d_select == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = pomdp_pbvi_update_gpu(pomdp, pbvi);
    if (rc != NOVA_SUCCESS) return rc;
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    return ws->eng.record(pbvi->d_pi, d_action, d_select, fn);
}

extern "C" int pomdp_pbvi_get_policy_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_pbvi_get_policy_gpu";
    if (pomdp == nullptr || pbvi == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (pomdp_alpha_vectors_initialize(policy, pomdp->n, pomdp->m, pomdp->r) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    const float *src = (pbvi->currentHorizon % 2u == 0u) ? pbvi->d_Gamma : pbvi->d_GammaPrime;
    int rc = d2h(policy->Gamma, src, (size_t)pomdp->r * pomdp->n * sizeof(float), fn, "Gamma");
    if (rc != NOVA_SUCCESS) return rc;
    return d2h(policy->pi, pbvi->d_pi, pomdp->r * sizeof(unsigned), fn, "pi");
}

extern "C" int pomdp_pbvi_execute_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_pbvi_execute_gpu";
    if (pomdp_shape_invalid(pomdp) || pomdp->d_S == nullptr || pomdp->d_T == nullptr || pomdp->d_O == nullptr ||
            pomdp->d_R == nullptr || pomdp->d_Z == nullptr || pomdp->d_B == nullptr || pbvi == nullptr ||
            pbvi->GammaInitial == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (pbvi->numThreads % 32 != 0) {
        NOVA_ERR(fn, "Invalid number of threads.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    int rc = pomdp_pbvi_initialize_gpu(pomdp, pbvi);
    if (rc != NOVA_SUCCESS) return rc;
    while (pbvi->currentHorizon < pomdp->horizon) {
        rc = pomdp_pbvi_update_gpu(pomdp, pbvi);
        if (rc != NOVA_SUCCESS) return rc;
    }
    rc = pomdp_pbvi_get_policy_gpu(pomdp, pbvi, policy);
    if (rc != NOVA_SUCCESS) return rc;
    return pomdp_pbvi_uninitialize_gpu(pomdp, pbvi);
}

extern "C" int pomdp_pbvi_set_graph_gpu(POMDPPBVIGPU *pbvi, unsigned int enable) {
    if (pbvi == nullptr) {
        NOVA_ERR("pomdp_pbvi_set_graph_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR("pomdp_pbvi_set_graph_gpu", "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    ws->eng.graphMode = enable != 0;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_set_scoring_gpu(POMDPPBVIGPU *pbvi, unsigned int mode) {
    if (pbvi == nullptr || (mode != NOVA_SCORING_EXACT && mode != NOVA_SCORING_BF16 && mode != NOVA_SCORING_FP16)) {
        NOVA_ERR("pomdp_pbvi_set_scoring_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR("pomdp_pbvi_set_scoring_gpu", "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (ws->eng.scoring != mode) {
        // Captured updates belong to the old mode (updates are synchronous,
        // so no replay is in flight).
        for (int d = 0; d < 2; d++) {
            if (ws->eng.graph[d]) cudaGraphExecDestroy(ws->eng.graph[d]);
            ws->eng.graph[d] = nullptr;
            ws->eng.graphSrc[d] = nullptr;
        }
    }
    ws->eng.scoring = mode;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_set_table_gpu(POMDPPBVIGPU *pbvi, unsigned int mode) {
    if (pbvi == nullptr || (mode != NOVA_PBVI_TABLE_AUTO && mode != NOVA_PBVI_TABLE_NEVER)) {
        NOVA_ERR("pomdp_pbvi_set_table_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR("pomdp_pbvi_set_table_gpu", "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    BackupEngine &e = ws->eng;
    const bool never = mode == NOVA_PBVI_TABLE_NEVER;
    if (e.tableNever != never) {
        // Captured updates read (or skip) the old table.
        for (int d = 0; d < 2; d++) {
            if (e.graph[d]) cudaGraphExecDestroy(e.graph[d]);
            e.graph[d] = nullptr;
            e.graphSrc[d] = nullptr;
        }
    }
    e.tableNever = never;
    if (never && e.Proj != nullptr) {
        cudaStreamSynchronize(e.stream);
        cudaFree(e.Proj);
        e.Proj = nullptr;
        e.projCap = 0;
        e.projCols = 0;
    }
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_get_stats_gpu(const POMDPPBVIGPU *pbvi, NovaPBVIStats *stats) {
    if (pbvi == nullptr || stats == nullptr) {
        NOVA_ERR("pomdp_pbvi_get_stats_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR("pomdp_pbvi_get_stats_gpu", "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    *stats = ws->eng.stats;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_row_detail_gpu(const POMDPPBVIGPU *pbvi, unsigned int *candidates,
                                         unsigned int *exactRows) {
    static const char *fn = "pomdp_pbvi_row_detail_gpu";
    if (pbvi == nullptr || candidates == nullptr || exactRows == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr || ws->eng.tc == nullptr || ws->eng.stats.tcGroups == 0) {
        NOVA_ERR(fn, "The solver's last update did not score on the tensor cores.");
        return NOVA_ERROR_INVALID_DATA;
    }
    return tc_row_detail(ws->eng, candidates, exactRows, fn);
}

extern "C" int pomdp_pbvi_value_gpu(const POMDP *pomdp, const POMDPPBVIGPU *pbvi, const float *b, double *Vb,
                                    unsigned int *a) {
    static const char *fn = "pomdp_pbvi_value_gpu";
    if (pomdp == nullptr || pbvi == nullptr || b == nullptr || Vb == nullptr || a == nullptr ||
            pbvi->d_Gamma == nullptr || pbvi->d_GammaPrime == nullptr || pbvi->d_pi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviGpuWorkspace *ws = pbvi_gpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = ensure_built(ws, pomdp, fn);
    if (rc != NOVA_SUCCESS) return rc;
    BackupEngine &e = ws->eng;
    const float *G = (pbvi->currentHorizon % 2u == 0u) ? pbvi->d_Gamma : pbvi->d_GammaPrime;
    if ((rc = h2d(e.bDense, b, pomdp->n * sizeof(float), fn, "the belief")) != NOVA_SUCCESS) return rc;
    row_dot_fp64_kernel<<<pomdp->r, 256, 0, e.stream>>>(G, pomdp->n, e.bDense, e.dotScratch);
    if ((rc = check_launch(fn, "FP64 belief values")) != NOVA_SUCCESS) return rc;
    argmax_fp64_kernel<<<1, 256, 0, e.stream>>>(e.dotScratch, pomdp->r, pbvi->d_pi, e.resultV, e.resultA);
    if ((rc = check_launch(fn, "FP64 belief argmax")) != NOVA_SUCCESS) return rc;
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(Vb, e.resultV, sizeof(double), fn, "the value")) != NOVA_SUCCESS) return rc;
    return d2h(a, e.resultA, sizeof(unsigned), fn, "the action");
}

// ===========================================================================
// Host-buffer PBVI (pomdp_pbvi_cpu.cpp): same engine, host arrays
// ===========================================================================

static PbviCpuWorkspace *pbvi_cpu_ws(const POMDPPBVICPU *pbvi) {
    std::lock_guard<std::mutex> lock(registry_mutex());
    return find_workspace<PbviCpuWorkspace>(pbvi);
}

extern "C" int pomdp_pbvi_uninitialize_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi) {
    (void)pomdp;
    if (pbvi == nullptr) {
        NOVA_ERR("pomdp_pbvi_uninitialize_cpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pbvi->currentHorizon = 0;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        registry().erase(pbvi);
    }
    delete[] pbvi->Gamma; pbvi->Gamma = nullptr;
    delete[] pbvi->GammaPrime; pbvi->GammaPrime = nullptr;
    delete[] pbvi->pi; pbvi->pi = nullptr;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_initialize_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi) {
    static const char *fn = "pomdp_pbvi_initialize_cpu";
    if (pomdp == nullptr || pbvi == nullptr || pomdp->n == 0 || pomdp->r == 0 || pbvi->GammaInitial == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pbvi->currentHorizon = 0;
    unsigned scoring = NOVA_SCORING_FP16;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *old = find_workspace<PbviCpuWorkspace>(pbvi);
        if (old != nullptr) {
            scoring = old->eng.scoring;
            const bool ownG = pbvi->Gamma == old->hostGamma, ownGP = pbvi->GammaPrime == old->hostGammaPrime,
                       ownPi = pbvi->pi == old->hostPi;
            registry().erase(pbvi);  // unpins the arrays it made
            if (ownG) { delete[] pbvi->Gamma; pbvi->Gamma = nullptr; }
            if (ownGP) { delete[] pbvi->GammaPrime; pbvi->GammaPrime = nullptr; }
            if (ownPi) { delete[] pbvi->pi; pbvi->pi = nullptr; }
        }
    }
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    // Host arrays as pomdp_pbvi_cpu.cpp:165-183.
    pbvi->Gamma = new float[rn];
    pbvi->GammaPrime = new float[rn];
    pbvi->pi = new unsigned int[pomdp->r];
    memcpy(pbvi->Gamma, pbvi->GammaInitial, rn * sizeof(float));
    memcpy(pbvi->GammaPrime, pbvi->GammaInitial, rn * sizeof(float));
    for (unsigned i = 0; i < pomdp->r; i++) pbvi->pi[i] = 0;
    std::unique_ptr<PbviCpuWorkspace> ws(new PbviCpuWorkspace());
    ws->eng.scoring = scoring;
    ws->hostGamma = pbvi->Gamma; ws->hostGammaPrime = pbvi->GammaPrime; ws->hostPi = pbvi->pi;
    // Page-locked in place (they stay new[] arrays, as the reference's
    // callers expect), so each update's host copies run at full link speed;
    // without it the copies are staged, with the same results.
    if (cudaHostRegister(pbvi->Gamma, rn * sizeof(float), cudaHostRegisterDefault) == cudaSuccess) {
        if (cudaHostRegister(pbvi->GammaPrime, rn * sizeof(float), cudaHostRegisterDefault) == cudaSuccess) {
            if (cudaHostRegister(pbvi->pi, pomdp->r * sizeof(unsigned), cudaHostRegisterDefault) == cudaSuccess) {
                ws->hostPinned = true;
            } else {
                cudaHostUnregister(pbvi->GammaPrime);
                cudaHostUnregister(pbvi->Gamma);
            }
        } else {
            cudaHostUnregister(pbvi->Gamma);
        }
    }
    cudaGetLastError();
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[pbvi] = std::move(ws);
    return NOVA_SUCCESS;
}

// The model is uploaded at the first update after initialize (the struct may
// be initialized before its arrays are filled) and reused afterwards.
static int pbvi_cpu_prepare(PbviCpuWorkspace *ws, const POMDP *pomdp, const char *fn) {
    if (ws->built) return NOVA_SUCCESS;
    if (pomdp->S == nullptr || pomdp->T == nullptr || pomdp->O == nullptr || pomdp->R == nullptr ||
            pomdp->Z == nullptr || pomdp->B == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    DevModel md;
    int rc = upload_model(ws, pomdp, &md, fn);
    if (rc != NOVA_SUCCESS) return rc;
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    if ((rc = dev_alloc(&ws->Gamma, rn, fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->GammaPrime, rn, fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->pi, pomdp->r, fn, "pi")) != NOVA_SUCCESS) return rc;
    if ((rc = ws->eng.build(md, fn)) != NOVA_SUCCESS) return rc;
    ws->built = true;
    return NOVA_SUCCESS;
}

// One backup with host arrays as the source of truth: upload the input set
// and pi, back up on the device, download the output set and pi (with the
// host's output set uploaded first when a belief keeps its row).
static int pbvi_cpu_step(PbviCpuWorkspace *ws, const POMDP *pomdp, POMDPPBVICPU *pbvi, const char *fn) {
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    const bool even = (pbvi->currentHorizon % 2u) == 0u;
    float *hsrc = even ? pbvi->Gamma : pbvi->GammaPrime;
    float *hdst = even ? pbvi->GammaPrime : pbvi->Gamma;
    int rc;
    if ((rc = h2d(ws->Gamma, hsrc, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->pi, pbvi->pi, pomdp->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
    if ((rc = ws->eng.backup_all(ws->Gamma, pomdp->r, ws->GammaPrime, ws->pi, fn)) != NOVA_SUCCESS) return rc;
    // The update writes every row of the output set except those of beliefs
    // no action of which beats the sentinel, so the host's output set is
    // uploaded only when such a belief exists; the update is then repeated
    // over it (the input set on the device is unchanged).
    unsigned kept = 0;
    if ((rc = ws->eng.count_kept(&kept, fn)) != NOVA_SUCCESS) return rc;
    if (kept != 0) {
        if ((rc = h2d(ws->GammaPrime, hdst, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(ws->pi, pbvi->pi, pomdp->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
        if ((rc = ws->eng.backup_all(ws->Gamma, pomdp->r, ws->GammaPrime, ws->pi, fn)) != NOVA_SUCCESS) return rc;
    }
    if ((rc = d2h(hdst, ws->GammaPrime, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(pbvi->pi, ws->pi, pomdp->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
    pbvi->currentHorizon++;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_update_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi) {
    static const char *fn = "pomdp_pbvi_update_cpu";
    if (pomdp_shape_invalid(pomdp) || pbvi == nullptr || pbvi->Gamma == nullptr || pbvi->GammaPrime == nullptr ||
            pbvi->pi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PbviCpuWorkspace *ws = pbvi_cpu_ws(pbvi);
    if (ws == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized (call pomdp_pbvi_initialize_cpu).");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = pbvi_cpu_prepare(ws, pomdp, fn);
    if (rc != NOVA_SUCCESS) return rc;
    return pbvi_cpu_step(ws, pomdp, pbvi, fn);
}

extern "C" int pomdp_pbvi_get_policy_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_pbvi_get_policy_cpu";
    if (pomdp == nullptr || pbvi == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments. Policy must be undefined.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (pomdp_alpha_vectors_initialize(policy, pomdp->n, pomdp->m, pomdp->r) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    const float *src = (pbvi->currentHorizon % 2u == 0u) ? pbvi->Gamma : pbvi->GammaPrime;
    memcpy(policy->Gamma, src, (size_t)pomdp->r * pomdp->n * sizeof(float));
    memcpy(policy->pi, pbvi->pi, pomdp->r * sizeof(unsigned));
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_execute_cpu(const POMDP *pomdp, POMDPPBVICPU *pbvi, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_pbvi_execute_cpu";
    if (pomdp_shape_invalid(pomdp) || pomdp->S == nullptr || pomdp->T == nullptr || pomdp->O == nullptr ||
            pomdp->R == nullptr || pomdp->Z == nullptr || pomdp->B == nullptr || pbvi == nullptr ||
            pbvi->GammaInitial == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = pomdp_pbvi_initialize_cpu(pomdp, pbvi);
    if (rc != NOVA_SUCCESS) return rc;
    PbviCpuWorkspace *ws = pbvi_cpu_ws(pbvi);
    if ((rc = pbvi_cpu_prepare(ws, pomdp, fn)) != NOVA_SUCCESS) return rc;
    // The whole horizon runs on the device; the sets come back once.
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    if ((rc = h2d(ws->Gamma, pbvi->Gamma, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->GammaPrime, pbvi->GammaPrime, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->pi, pbvi->pi, pomdp->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
    while (pbvi->currentHorizon < pomdp->horizon) {
        const bool even = (pbvi->currentHorizon % 2u) == 0u;
        rc = ws->eng.backup_all(even ? ws->Gamma : ws->GammaPrime, pomdp->r, even ? ws->GammaPrime : ws->Gamma,
                                ws->pi, fn);
        if (rc != NOVA_SUCCESS) return rc;
        pbvi->currentHorizon++;
    }
    if ((rc = d2h(pbvi->Gamma, ws->Gamma, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(pbvi->GammaPrime, ws->GammaPrime, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(pbvi->pi, ws->pi, pomdp->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
    rc = pomdp_pbvi_get_policy_cpu(pomdp, pbvi, policy);
    if (rc != NOVA_SUCCESS) return rc;
    return pomdp_pbvi_uninitialize_cpu(pomdp, pbvi);
}
