// nova-gb300: V(b) and the policy's action for many beliefs at once.
//
// For each belief b (dense, n states) the reference evaluates
// (pomdp_alpha_vectors.cpp:52-79)
//
//   V_i = sum_s fl(Gamma_i(s) * b(s))   (added in state order, FP32)
//   V(b) = max_i V_i                     (from -1e10, strict '<': lowest i on ties)
//   a(b) = pi[argmax]
//
// Here the V_i of a tile of beliefs against a tile of alphas are one
// register-tiled FP32 product (beliefs x states) . (states x alphas): every
// thread owns a 4 x 4 block of (belief, alpha) sums and adds its terms in
// state order with separately rounded products and sums, so each V_i has the
// reference's bits; tiles of 32 states of both operands are staged in shared
// memory. Two alphas per instruction: f32x2 products, summed with the exact
// f32x2 form (fma of the product by a run-time 1.0). The epilogue keeps, per belief and alpha tile, the best V and its
// lowest index; a second pass merges the tiles in alpha order.

#include "common.h"

#include <nova/constants.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>
#include <nova/nova_gb300.h>

using nova::POMDPAlphaVectors;

namespace nova_gb300 {
namespace {

constexpr unsigned TB = 64;       // beliefs per tile
constexpr unsigned TA = 64;       // alphas per tile
constexpr unsigned TK = 32;       // states per shared-memory stage
constexpr unsigned kThreads = 256;
constexpr unsigned kNone = 0xffffffffu;

// Partial maxima: part[belief][alphaTile] = (value, alpha index).
__global__ void __launch_bounds__(kThreads) value_tiles_kernel(const float *__restrict__ G, unsigned r, unsigned n,
                                                               const float *__restrict__ Bd, unsigned count,
                                                               float *__restrict__ partV,
                                                               unsigned *__restrict__ partI, unsigned aTiles,
                                                               float one) {
    // State-major tiles, belief (alpha) contiguous; rows padded by 4 floats so
    // the staging stores spread over the banks and rows stay 16-byte aligned.
    __shared__ __align__(16) float sB[TK][TB + 4];
    __shared__ __align__(16) float sG[TK][TA + 4];
    const unsigned tid = threadIdx.x;
    const unsigned tx = tid % 16, ty = tid / 16;  // alpha group, belief group
    const unsigned b0 = blockIdx.y * TB, a0 = blockIdx.x * TA;
    const unsigned long long one2 = pack_f32x2(one, one);
    unsigned long long acc2[4][2];  // (alpha 4tx+2p, 4tx+2p+1) per belief row i
#pragma unroll
    for (int i = 0; i < 4; i++) { acc2[i][0] = 0ull; acc2[i][1] = 0ull; }
    for (unsigned k0 = 0; k0 < n; k0 += TK) {
        // Stage TK states of TB beliefs and TA alphas (zeros past the ends,
        // which are never added: the state loop stops at n, and rows past
        // count or r are not reported).
        // Eight threads read 32 consecutive states of one row (four each).
        for (unsigned e = tid; e < TB * (TK / 4); e += kThreads) {
            const unsigned bb = e / (TK / 4), k4 = e % (TK / 4);
            const unsigned bi = b0 + bb;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned s = k0 + 4 * k4 + q;
                sB[4 * k4 + q][bb] = (s < n && bi < count) ? Bd[(size_t)bi * n + s] : 0.0f;
            }
        }
        for (unsigned e = tid; e < TA * (TK / 4); e += kThreads) {
            const unsigned aa = e / (TK / 4), k4 = e % (TK / 4);
            const unsigned ai = a0 + aa;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned s = k0 + 4 * k4 + q;
                sG[4 * k4 + q][aa] = (s < n && ai < r) ? G[(size_t)ai * n + s] : 0.0f;
            }
        }
        __syncthreads();
        const unsigned kEnd = min(TK, n - k0);
        for (unsigned kk = 0; kk < kEnd; kk++) {
            const float4 bv = *reinterpret_cast<const float4 *>(&sB[kk][4 * ty]);
            const ulonglong2 gv = *reinterpret_cast<const ulonglong2 *>(&sG[kk][4 * tx]);
            const float bq[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const unsigned long long bb = pack_f32x2(bq[i], bq[i]);
                acc2[i][0] = fma_f32x2(mul_f32x2(gv.x, bb), one2, acc2[i][0]);
                acc2[i][1] = fma_f32x2(mul_f32x2(gv.y, bb), one2, acc2[i][1]);
            }
        }
        __syncthreads();
    }
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = f32x2_part(acc2[i][j / 2], j & 1);
    // Best alpha of this tile per belief: the 16 threads of a belief group
    // hold 4 alphas each; reduce with shuffles (max value, then lowest index).
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float best = NOVA_FLT_MIN;
        unsigned bi = kNone;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const unsigned ai = a0 + 4 * tx + j;
            if (ai < r && best < acc[i][j]) { best = acc[i][j]; bi = ai; }
        }
        for (int off = 8; off > 0; off >>= 1) {
            const float ov = __shfl_down_sync(0xffffffffu, best, off, 16);
            const unsigned oi = __shfl_down_sync(0xffffffffu, bi, off, 16);
            if (oi != kNone && (bi == kNone || ov > best || (ov == best && oi < bi))) { best = ov; bi = oi; }
        }
        const unsigned belief = b0 + 4 * ty + i;
        if (tx == 0 && belief < count) {
            partV[(size_t)belief * aTiles + blockIdx.x] = best;
            partI[(size_t)belief * aTiles + blockIdx.x] = bi;
        }
    }
}

__global__ void value_merge_kernel(unsigned count, unsigned aTiles, const float *__restrict__ partV,
                                   const unsigned *__restrict__ partI, const unsigned *__restrict__ pi,
                                   float *__restrict__ V, unsigned *__restrict__ act) {
    const unsigned b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count) return;
    float best = NOVA_FLT_MIN;
    unsigned bi = kNone;
    for (unsigned t = 0; t < aTiles; t++) {
        const unsigned i = partI[(size_t)b * aTiles + t];
        const float v = partV[(size_t)b * aTiles + t];
        if (i != kNone && best < v) { best = v; bi = i; }
    }
    V[b] = best;
    act[b] = bi == kNone ? 0u : pi[bi];
}

}  // namespace

static int value_batched(const float *dG, const unsigned *dPi, unsigned r, unsigned n, const float *dB,
                         unsigned count, float *dV, unsigned *dA, const char *fn) {
    const unsigned aTiles = ceil_div(r, TA);
    float *partV = nullptr;
    unsigned *partI = nullptr;
    int rc;
    if ((rc = dev_alloc(&partV, (size_t)count * aTiles, fn, "the partial maxima")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&partI, (size_t)count * aTiles, fn, "the partial arg-maxima")) != NOVA_SUCCESS) {
        cudaFree(partV);
        return rc;
    }
    value_tiles_kernel<<<dim3(aTiles, ceil_div(count, TB)), kThreads>>>(dG, r, n, dB, count, partV, partI, aTiles,
                                                                        1.0f);
    rc = check_launch(fn, "belief values");
    if (rc == NOVA_SUCCESS) {
        value_merge_kernel<<<ceil_div(count, 256), 256>>>(count, aTiles, partV, partI, dPi, dV, dA);
        rc = check_launch(fn, "belief arg-maxima");
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    cudaFree(partV);
    cudaFree(partI);
    return rc;
}

}  // namespace nova_gb300

using namespace nova_gb300;

extern "C" int pomdp_alpha_vectors_value_batched_gpu(const float *d_Gamma, const unsigned int *d_pi, unsigned int r,
                                                     unsigned int n, const float *d_B, unsigned int count,
                                                     float *d_V, unsigned int *d_a) {
    static const char *fn = "pomdp_alpha_vectors_value_batched_gpu";
    if (d_Gamma == nullptr || d_pi == nullptr || d_B == nullptr || d_V == nullptr || d_a == nullptr || r == 0 ||
            n == 0 || count == 0) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    return value_batched(d_Gamma, d_pi, r, n, d_B, count, d_V, d_a, fn);
}

extern "C" int pomdp_alpha_vectors_value_and_action_batched(const POMDPAlphaVectors *policy, const float *B,
                                                            unsigned int count, float *V, unsigned int *a) {
    static const char *fn = "pomdp_alpha_vectors_value_and_action_batched";
    if (policy == nullptr || policy->n == 0 || policy->m == 0 || policy->r == 0 || policy->Gamma == nullptr ||
            policy->pi == nullptr || B == nullptr || V == nullptr || a == nullptr || count == 0) {
        NOVA_ERR(fn, "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned r = policy->r, n = policy->n;
    float *dG = nullptr, *dB = nullptr, *dV = nullptr;
    unsigned *dPi = nullptr, *dA = nullptr;
    struct Free {
        float *&g, *&b, *&v; unsigned *&p, *&a;
        ~Free() { cudaFree(g); cudaFree(b); cudaFree(v); cudaFree(p); cudaFree(a); }
    } guard{dG, dB, dV, dPi, dA};
    int rc;
    if ((rc = dev_alloc(&dG, (size_t)r * n, fn, "the alpha-vectors")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dPi, r, fn, "the policy actions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dB, (size_t)count * n, fn, "the beliefs")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dV, count, fn, "the values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&dA, count, fn, "the actions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(dG, policy->Gamma, (size_t)r * n * sizeof(float), fn, "the alpha-vectors")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(dPi, policy->pi, r * sizeof(unsigned), fn, "the policy actions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(dB, B, (size_t)count * n * sizeof(float), fn, "the beliefs")) != NOVA_SUCCESS) return rc;
    if ((rc = value_batched(dG, dPi, r, n, dB, count, dV, dA, fn)) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(V, dV, count * sizeof(float), fn, "the values")) != NOVA_SUCCESS) return rc;
    return d2h(a, dA, count * sizeof(unsigned), fn, "the actions");
}
