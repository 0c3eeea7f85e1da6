// nova-gb300: Perseus on the GB300 (pomdp_perseus_*_gpu, new) and the
// host-buffer entry points pomdp_perseus_*_cpu.
//
// One update (pomdp_perseus_cpu.cpp:312-429):
//   * draw a belief from B~ with rand() on the host (the reference formula);
//   * back it up against V_n = Gamma[0, rGamma) with the exact-order engine
//     (dedup + scoring + assembly of pbvi.cu, restricted to one belief);
//   * keep the new alpha if it does not lose value at the belief, else copy
//     the belief's best old alpha (pomdp_perseus_cpu.cpp:367-374);
//   * rebuild B~ = {i : V_{n+1}(b_i) < V_n(b_i)} (pomdp_perseus_cpu.cpp:387-402).
// V_n(b_i) is constant within a horizon step and is computed once per step;
// V_{n+1}(b_i) is a running maximum updated with the one new alpha, which is
// exact because only the maximum value (not its index) enters the test.

#include "pbvi.h"

#include <cstdlib>
#include <vector>

#include <nova/constants.h>
#include <nova/pomdp/algorithms/pomdp_perseus_cpu.h>
#include <nova/pomdp/algorithms/pomdp_perseus_gpu.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

using nova::POMDP;
using nova::POMDPPerseusCPU;
using nova::POMDPPerseusGPU;
using nova::POMDPAlphaVectors;

namespace nova_gb300 {

constexpr unsigned kNoneP = 0xffffffffu;

// b_i . alpha over the belief support in the order of
// pomdp_perseus_compute_b_dot_alpha_cpu (pomdp_perseus_cpu.cpp:37-50).
__device__ __forceinline__ float belief_dot(const DevModel &md, unsigned Li, unsigned i, const float *alpha) {
    float acc = 0.0f;
    for (unsigned k = 0; k < Li; k++) {
        const int s = md.Z[(size_t)i * md.rz + k];
        acc = fadd(acc, fmul(md.B[(size_t)i * md.rz + k], alpha[s]));
    }
    return acc;
}

// V(b_i) = max over rows [0, rows) of b_i . G_j, first maximiser
// (pomdp_perseus_compute_Vb_cpu, pomdp_perseus_cpu.cpp:53-68). One block per
// belief. idxOut may be null.
__global__ void perseus_vb_kernel(DevModel md, const unsigned *__restrict__ suppLen, const float *__restrict__ G,
                                  unsigned rows, float *__restrict__ vOut, unsigned *__restrict__ idxOut) {
    const unsigned i = blockIdx.x;
    const unsigned Li = suppLen[i];
    float best = NOVA_FLT_MIN;
    unsigned bj = kNoneP;
    for (unsigned j = threadIdx.x; j < rows; j += blockDim.x) {
        const float d = belief_dot(md, Li, i, G + (size_t)j * md.n);
        if (best < d) { best = d; bj = j; }
    }
    __shared__ float sv[256];
    __shared__ unsigned si[256];
    sv[threadIdx.x] = best; si[threadIdx.x] = bj;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = NOVA_FLT_MIN;
        unsigned bi = kNoneP;
        for (unsigned t = 0; t < blockDim.x; t++) {
            if (si[t] == kNoneP) continue;
            if (bi == kNoneP || sv[t] > b || (sv[t] == b && si[t] < bi)) { b = sv[t]; bi = si[t]; }
        }
        vOut[i] = b;
        // The reference's caller starts alphaPrimeIndex at 0 (pomdp_perseus_cpu.cpp:361).
        if (idxOut) idxOut[i] = bi == kNoneP ? 0u : bi;
    }
}

// Keep the new alpha or copy the belief's best old one, into slot `slot`.
__global__ void perseus_commit_kernel(DevModel md, const unsigned *__restrict__ suppLen, unsigned bIndex,
                                      const float *__restrict__ alpha, const unsigned *__restrict__ alphaAction,
                                      const float *__restrict__ vnb, const unsigned *__restrict__ vnbIdx,
                                      const float *__restrict__ G, const unsigned *__restrict__ pi,
                                      float *__restrict__ Gp, unsigned *__restrict__ piP, unsigned slot) {
    __shared__ int keepNew;
    if (threadIdx.x == 0) {
        const float bDotAlpha = belief_dot(md, suppLen[bIndex], bIndex, alpha);
        keepNew = bDotAlpha >= vnb[bIndex] ? 1 : 0;
        const unsigned act = *alphaAction == kNoneP ? 0u : *alphaAction;
        piP[slot] = keepNew ? act : pi[vnbIdx[bIndex]];
    }
    __syncthreads();
    const float *srcRow = keepNew ? alpha : G + (size_t)vnbIdx[bIndex] * md.n;
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) Gp[(size_t)slot * md.n + s] = srcRow[s];
}

// V_{n+1}(b_i) <- max(V_{n+1}(b_i), b_i . newRow) with the reference's strict '<'.
__global__ void perseus_raise_kernel(DevModel md, const unsigned *__restrict__ suppLen, const float *__restrict__ row,
                                     float *__restrict__ vnp1b) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= md.r) return;
    const float d = belief_dot(md, suppLen[i], i, row);
    if (vnp1b[i] < d) vnp1b[i] = d;
}

// B~ = {i : V_{n+1}(b_i) < V_n(b_i)} in increasing i (single block).
__global__ void __launch_bounds__(1024) perseus_btilde_kernel(unsigned r, const float *__restrict__ vnb,
                                                              const float *__restrict__ vnp1b,
                                                              unsigned *__restrict__ out, unsigned *__restrict__ count) {
    __shared__ unsigned warpSums[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (unsigned base = 0; base < r; base += blockDim.x) {
        const unsigned i = base + threadIdx.x;
        const unsigned flag = (i < r && vnp1b[i] < vnb[i]) ? 1u : 0u;
        unsigned v = flag;
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
            warpSums[lane] = w;
        }
        __syncthreads();
        const unsigned pos = carry + (warp > 0 ? warpSums[warp - 1] : 0u) + v - flag;
        if (flag) out[pos] = i;
        __syncthreads();
        if (threadIdx.x == 0) carry += warpSums[(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

__global__ void fill_float_kernel(float *p, unsigned count, float v) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) p[t] = v;
}

// Device-side Perseus state shared by the _gpu and _cpu front ends.
struct PerseusCore {
    BackupEngine eng;
    bool built = false;
    unsigned *vnbIdx = nullptr;
    // Validity of the per-horizon-step caches (V_n values, V_n dedup).
    bool cacheValid = false;
    unsigned cacheHorizon = 0;
    unsigned nU = 0;
    ~PerseusCore() { cudaFree(vnbIdx); }

    int build(const DevModel &md, const char *fn) {
        int rc = eng.build(md, fn);
        if (rc != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&eng.vnb, md.r, fn, "V_n(b)")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&eng.vnp1b, md.r, fn, "V_n+1(b)")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&eng.btilde, md.r, fn, "B~")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&vnbIdx, md.r, fn, "argmax V_n(b)")) != NOVA_SUCCESS) return rc;
        built = true;
        return NOVA_SUCCESS;
    }

    // Per-step caches: V_n(b_i) with maximisers, the dedup of V_n, and
    // V_{n+1}(b_i) over the rows already in Gamma'.
    int refresh(const float *G, unsigned rGamma, const float *Gp, unsigned rGammaPrime, const char *fn) {
        const DevModel &md = eng.md;
        int rc;
        if (rGamma > 0) {
            perseus_vb_kernel<<<md.r, 256, 0, eng.stream>>>(md, eng.suppLen, G, rGamma, eng.vnb, vnbIdx);
        } else {
            fill_float_kernel<<<ceil_div(md.r, 256), 256, 0, eng.stream>>>(eng.vnb, md.r, NOVA_FLT_MIN);
            cudaMemsetAsync(vnbIdx, 0, md.r * sizeof(unsigned), eng.stream);
        }
        if ((rc = check_launch(fn, "V_n(b)")) != NOVA_SUCCESS) return rc;
        if (rGammaPrime > 0)
            perseus_vb_kernel<<<md.r, 256, 0, eng.stream>>>(md, eng.suppLen, Gp, rGammaPrime, eng.vnp1b, nullptr);
        else
            fill_float_kernel<<<ceil_div(md.r, 256), 256, 0, eng.stream>>>(eng.vnp1b, md.r, NOVA_FLT_MIN);
        if ((rc = check_launch(fn, "V_n+1(b)")) != NOVA_SUCCESS) return rc;
        nU = 0;
        if (rGamma > 0 && (rc = eng.dedup(G, rGamma, &nU, fn)) != NOVA_SUCCESS) return rc;
        cacheValid = true;
        return NOVA_SUCCESS;
    }

    // One Perseus update. G/pi: V_n and its actions (rGamma rows);
    // Gp/piP: V_{n+1} (rGammaPrime rows). Host bookkeeping by reference.
    // newSlot receives the row index written into Gp.
    int update(const float *G, const unsigned *pi, float *Gp, unsigned *piP, unsigned &currentHorizon,
               unsigned &rGamma, unsigned &rGammaPrime, unsigned &rTilde, unsigned *BTilde, unsigned *newSlot,
               const char *fn) {
        const DevModel &md = eng.md;
        int rc;
        if (!cacheValid || cacheHorizon != currentHorizon) {
            if ((rc = refresh(G, rGamma, Gp, rGammaPrime, fn)) != NOVA_SUCCESS) return rc;
            cacheHorizon = currentHorizon;
        }
        // Belief draw of pomdp_perseus_cpu.cpp:340-341. When rand() rounds
        // to RAND_MAX the index equals rTilde and the reference reads the
        // stale entry there; beyond the array it is clamped to the last one.
        unsigned bTildeIndex = (unsigned)((float)rand() / (float)RAND_MAX * (float)rTilde);
        if (bTildeIndex >= md.r) bTildeIndex = md.r - 1;
        const unsigned bIndex = BTilde[bTildeIndex];
        if (bIndex >= md.r) {
            NOVA_ERR(fn, "Invalid belief index in BTilde.");
            return NOVA_ERROR_INVALID_DATA;
        }
        if (rGammaPrime + 1 > md.r) {
            NOVA_ERR(fn, "Out of memory. Too many alpha-vectors added.");
            return NOVA_ERROR_OUT_OF_MEMORY;
        }
        // Backup of belief bIndex against V_n.
        if (rGamma == 0) {
            // The reference's best-alpha index is never assigned when V_n is
            // empty (pomdp_perseus_cpu.cpp:78-84); row 0 is used here.
            cudaMemsetAsync(eng.jstar + (size_t)bIndex * md.m * md.z, 0, (size_t)md.m * md.z * sizeof(unsigned),
                            eng.stream);
        } else {
            if ((rc = eng.fill_items(bIndex * md.m, md.m, fn)) != NOVA_SUCCESS) return rc;
            if ((rc = eng.exact_score(eng.items, md.m, nU, fn)) != NOVA_SUCCESS) return rc;
        }
        if ((rc = eng.assemble(G, nullptr, nullptr, (int)bIndex, eng.rowScratch, eng.resultA, fn)) != NOVA_SUCCESS)
            return rc;
        const unsigned slot = rGammaPrime;
        perseus_commit_kernel<<<1, 256, 0, eng.stream>>>(md, eng.suppLen, bIndex, eng.rowScratch, eng.resultA,
                                                         eng.vnb, vnbIdx, G, pi, Gp, piP, slot);
        if ((rc = check_launch(fn, "Perseus commit")) != NOVA_SUCCESS) return rc;
        rGammaPrime++;
        *newSlot = slot;
        perseus_raise_kernel<<<ceil_div(md.r, 256), 256, 0, eng.stream>>>(md, eng.suppLen, Gp + (size_t)slot * md.n,
                                                                          eng.vnp1b);
        if ((rc = check_launch(fn, "V_n+1(b) update")) != NOVA_SUCCESS) return rc;
        perseus_btilde_kernel<<<1, 1024, 0, eng.stream>>>(md.r, eng.vnb, eng.vnp1b, eng.btilde, eng.itemCount);
        if ((rc = check_launch(fn, "B~")) != NOVA_SUCCESS) return rc;
        unsigned count = 0;
        if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;
        if ((rc = d2h(&count, eng.itemCount, sizeof(unsigned), fn, "|B~|")) != NOVA_SUCCESS) return rc;
        if (count > 0 && (rc = d2h(BTilde, eng.btilde, count * sizeof(unsigned), fn, "B~")) != NOVA_SUCCESS)
            return rc;
        rTilde = count;
        if (rTilde == 0) {
            // pomdp_perseus_cpu.cpp:405-426
            currentHorizon++;
            rGamma = 0;
            rTilde = md.r;
            for (unsigned i = 0; i < md.r; i++) BTilde[i] = i;
            cacheValid = false;
            return NOVA_CONVERGED;
        }
        return NOVA_SUCCESS;
    }
};

struct PerseusGpuWorkspace : Workspace {
    PerseusCore core;
    const void *modelKey[6] = {};
    float *d_Gamma = nullptr, *d_GammaPrime = nullptr;
    unsigned *d_pi = nullptr, *d_piPrime = nullptr;
    unsigned *hostBTilde = nullptr;
    ~PerseusGpuWorkspace() override {
        cudaDeviceSynchronize();
        cudaFree(d_Gamma); cudaFree(d_GammaPrime); cudaFree(d_pi); cudaFree(d_piPrime);
    }
};

struct PerseusCpuWorkspace : Workspace {
    PerseusCore core;
    int *S = nullptr; float *T = nullptr, *O = nullptr, *R = nullptr; int *Z = nullptr; float *B = nullptr;
    float *Gamma = nullptr, *GammaPrime = nullptr;
    unsigned *pi = nullptr, *piPrime = nullptr;
    ~PerseusCpuWorkspace() override {
        cudaDeviceSynchronize();
        cudaFree(S); cudaFree(T); cudaFree(O); cudaFree(R); cudaFree(Z); cudaFree(B);
        cudaFree(Gamma); cudaFree(GammaPrime); cudaFree(pi); cudaFree(piPrime);
    }
};

static bool perseus_shape_invalid(const POMDP *p) {
    return p == nullptr || p->n == 0 || p->ns == 0 || p->m == 0 || p->z == 0 || p->r == 0 || p->rz == 0 ||
           p->gamma < 0.0f || p->gamma > 1.0f || p->horizon < 1;
}

}  // namespace nova_gb300

using namespace nova_gb300;

// ===========================================================================
// Device-buffer Perseus (new)
// ===========================================================================

static PerseusGpuWorkspace *perseus_gpu_ws(const POMDPPerseusGPU *per) {
    std::lock_guard<std::mutex> lock(registry_mutex());
    return find_workspace<PerseusGpuWorkspace>(per);
}

extern "C" int pomdp_perseus_uninitialize_gpu(const POMDP *pomdp, POMDPPerseusGPU *per) {
    (void)pomdp;
    if (per == nullptr) {
        NOVA_ERR("pomdp_perseus_uninitialize_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    per->currentHorizon = 0;
    per->rGamma = 0; per->rGammaPrime = 0; per->rTilde = 0;
    std::lock_guard<std::mutex> lock(registry_mutex());
    auto *ws = find_workspace<PerseusGpuWorkspace>(per);
    if (ws != nullptr) {
        if (per->BTilde == ws->hostBTilde) { delete[] per->BTilde; per->BTilde = nullptr; }
        per->d_Gamma = nullptr; per->d_GammaPrime = nullptr; per->d_pi = nullptr; per->d_piPrime = nullptr;
        registry().erase(per);
    }
    return NOVA_SUCCESS;
}

extern "C" int pomdp_perseus_initialize_gpu(const POMDP *pomdp, POMDPPerseusGPU *per) {
    static const char *fn = "pomdp_perseus_initialize_gpu";
    if (pomdp == nullptr || per == nullptr || pomdp->n == 0 || pomdp->r == 0 || per->GammaInitial == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *old = find_workspace<PerseusGpuWorkspace>(per);
        if (old != nullptr) {
            if (per->BTilde == old->hostBTilde) { delete[] per->BTilde; per->BTilde = nullptr; }
            registry().erase(per);
        }
    }
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    std::unique_ptr<PerseusGpuWorkspace> ws(new PerseusGpuWorkspace());
    int rc;
    if ((rc = dev_alloc(&ws->d_Gamma, rn, fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_GammaPrime, rn, fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_pi, pomdp->r, fn, "pi")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_piPrime, pomdp->r, fn, "pi (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->d_Gamma, per->GammaInitial, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->d_GammaPrime, per->GammaInitial, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS)
        return rc;
    cudaMemset(ws->d_pi, 0, pomdp->r * sizeof(unsigned));
    cudaMemset(ws->d_piPrime, 0, pomdp->r * sizeof(unsigned));
    // pomdp_perseus_cpu.cpp:183-219: empty V_n and V_{n+1}, B~ = B.
    per->currentHorizon = 0;
    per->rGamma = 0;
    per->rGammaPrime = 0;
    per->rTilde = pomdp->r;
    per->BTilde = new unsigned int[pomdp->r];
    for (unsigned i = 0; i < pomdp->r; i++) per->BTilde[i] = i;
    ws->hostBTilde = per->BTilde;
    per->d_Gamma = ws->d_Gamma; per->d_GammaPrime = ws->d_GammaPrime;
    per->d_pi = ws->d_pi; per->d_piPrime = ws->d_piPrime;
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[per] = std::move(ws);
    return NOVA_SUCCESS;
}

extern "C" int pomdp_perseus_update_gpu(const POMDP *pomdp, POMDPPerseusGPU *per) {
    static const char *fn = "pomdp_perseus_update_gpu";
    if (perseus_shape_invalid(pomdp) || per == nullptr || pomdp->d_S == nullptr || pomdp->d_T == nullptr ||
            pomdp->d_O == nullptr || pomdp->d_R == nullptr || pomdp->d_Z == nullptr || pomdp->d_B == nullptr ||
            per->BTilde == nullptr || per->d_Gamma == nullptr || per->d_GammaPrime == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PerseusGpuWorkspace *ws = perseus_gpu_ws(per);
    if (ws == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized (call pomdp_perseus_initialize_gpu).");
        return NOVA_ERROR_INVALID_DATA;
    }
    const void *key[6] = {pomdp->d_S, pomdp->d_T, pomdp->d_O, pomdp->d_R, pomdp->d_Z, pomdp->d_B};
    if (!ws->core.built || memcmp(key, ws->modelKey, sizeof(key)) != 0) {
        if (ws->core.built) {
            NOVA_ERR(fn, "The device model changed during a Perseus solve.");
            return NOVA_ERROR_INVALID_DATA;
        }
        DevModel md;
        md.n = pomdp->n; md.ns = pomdp->ns; md.m = pomdp->m; md.z = pomdp->z; md.r = pomdp->r;
        md.rz = pomdp->rz; md.gamma = pomdp->gamma;
        md.S = pomdp->d_S; md.T = pomdp->d_T; md.O = pomdp->d_O; md.R = pomdp->d_R; md.Z = pomdp->d_Z;
        md.B = pomdp->d_B;
        int rc = ws->core.build(md, fn);
        if (rc != NOVA_SUCCESS) return rc;
        memcpy(ws->modelKey, key, sizeof(key));
    }
    const bool even = (per->currentHorizon % 2u) == 0u;
    unsigned slot = 0;
    if (even)
        return ws->core.update(per->d_Gamma, per->d_pi, per->d_GammaPrime, per->d_piPrime, per->currentHorizon,
                               per->rGamma, per->rGammaPrime, per->rTilde, per->BTilde, &slot, fn);
    return ws->core.update(per->d_GammaPrime, per->d_piPrime, per->d_Gamma, per->d_pi, per->currentHorizon,
                           per->rGammaPrime, per->rGamma, per->rTilde, per->BTilde, &slot, fn);
}

extern "C" int pomdp_perseus_get_policy_gpu(const POMDP *pomdp, POMDPPerseusGPU *per, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_perseus_get_policy_gpu";
    if (pomdp == nullptr || per == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const bool even = (per->currentHorizon % 2u) == 0u;
    const unsigned rows = even ? per->rGamma : per->rGammaPrime;
    if (pomdp_alpha_vectors_initialize(policy, pomdp->n, pomdp->m, rows) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    int rc = d2h(policy->Gamma, even ? per->d_Gamma : per->d_GammaPrime, (size_t)rows * pomdp->n * sizeof(float),
                 fn, "Gamma");
    if (rc != NOVA_SUCCESS) return rc;
    return d2h(policy->pi, even ? per->d_pi : per->d_piPrime, rows * sizeof(unsigned), fn, "pi");
}

extern "C" int pomdp_perseus_execute_gpu(const POMDP *pomdp, POMDPPerseusGPU *per, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_perseus_execute_gpu";
    if (perseus_shape_invalid(pomdp) || pomdp->d_S == nullptr || pomdp->d_T == nullptr || pomdp->d_O == nullptr ||
            pomdp->d_R == nullptr || pomdp->d_Z == nullptr || pomdp->d_B == nullptr || per == nullptr ||
            per->GammaInitial == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (per->numThreads % 32 != 0) {
        NOVA_ERR(fn, "Invalid number of threads.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    int rc = pomdp_perseus_initialize_gpu(pomdp, per);
    if (rc != NOVA_SUCCESS) return rc;
    while (per->currentHorizon < pomdp->horizon) {
        rc = NOVA_SUCCESS;
        while (rc != NOVA_CONVERGED) {
            rc = pomdp_perseus_update_gpu(pomdp, per);
            if (rc != NOVA_CONVERGED && rc != NOVA_SUCCESS) return rc;
        }
    }
    rc = pomdp_perseus_get_policy_gpu(pomdp, per, policy);
    if (rc != NOVA_SUCCESS) return rc;
    return pomdp_perseus_uninitialize_gpu(pomdp, per);
}

// ===========================================================================
// Host-buffer Perseus (pomdp_perseus_cpu.cpp)
// ===========================================================================

static PerseusCpuWorkspace *perseus_cpu_ws(const POMDPPerseusCPU *per) {
    std::lock_guard<std::mutex> lock(registry_mutex());
    return find_workspace<PerseusCpuWorkspace>(per);
}

extern "C" int pomdp_perseus_uninitialize_cpu(const POMDP *pomdp, POMDPPerseusCPU *per) {
    (void)pomdp;
    if (per == nullptr) {
        NOVA_ERR("pomdp_perseus_uninitialize_cpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        registry().erase(per);
    }
    // pomdp_perseus_cpu.cpp:273-309
    per->currentHorizon = 0;
    delete[] per->Gamma; per->Gamma = nullptr; per->rGamma = 0;
    delete[] per->GammaPrime; per->GammaPrime = nullptr; per->rGammaPrime = 0;
    delete[] per->pi; per->pi = nullptr;
    delete[] per->piPrime; per->piPrime = nullptr;
    delete[] per->BTilde; per->BTilde = nullptr; per->rTilde = 0;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_perseus_initialize_cpu(const POMDP *pomdp, POMDPPerseusCPU *per) {
    static const char *fn = "pomdp_perseus_initialize_cpu";
    if (pomdp == nullptr || per == nullptr || pomdp->n == 0 || pomdp->r == 0 || per->GammaInitial == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        registry().erase(per);
    }
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    // Host arrays of pomdp_perseus_cpu.cpp:183-219.
    per->currentHorizon = 0;
    per->Gamma = new float[rn];
    per->GammaPrime = new float[rn];
    per->pi = new unsigned int[pomdp->r];
    per->piPrime = new unsigned int[pomdp->r];
    memcpy(per->Gamma, per->GammaInitial, rn * sizeof(float));
    memcpy(per->GammaPrime, per->GammaInitial, rn * sizeof(float));
    for (unsigned i = 0; i < pomdp->r; i++) { per->pi[i] = 0; per->piPrime[i] = 0; }
    per->rGamma = 0;
    per->rGammaPrime = 0;
    per->rTilde = pomdp->r;
    per->BTilde = new unsigned int[pomdp->r];
    for (unsigned i = 0; i < pomdp->r; i++) per->BTilde[i] = i;
    std::unique_ptr<PerseusCpuWorkspace> ws(new PerseusCpuWorkspace());
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[per] = std::move(ws);
    return NOVA_SUCCESS;
}

// Model and solver arrays are uploaded at the first update; afterwards the
// device copies are authoritative and each update writes the one new alpha
// row and action back into the host arrays.
static int perseus_cpu_prepare(PerseusCpuWorkspace *ws, const POMDP *p, POMDPPerseusCPU *per, const char *fn) {
    if (ws->core.built) return NOVA_SUCCESS;
    if (p->S == nullptr || p->T == nullptr || p->O == nullptr || p->R == nullptr || p->Z == nullptr ||
            p->B == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const size_t nms = (size_t)p->n * p->m * p->ns, mnz = (size_t)p->m * p->n * p->z, nm = (size_t)p->n * p->m,
                 rrz = (size_t)p->r * p->rz, rn = (size_t)p->r * p->n;
    int rc;
    if ((rc = dev_alloc(&ws->S, nms, fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->T, nms, fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->O, mnz, fn, "the observation transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->R, nm, fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->Z, rrz, fn, "the non-zero belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->B, rrz, fn, "the belief points")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->Gamma, rn, fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->GammaPrime, rn, fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->pi, p->r, fn, "pi")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->piPrime, p->r, fn, "pi (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->S, p->S, nms * sizeof(int), fn, "the successor states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->T, p->T, nms * sizeof(float), fn, "the state transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->O, p->O, mnz * sizeof(float), fn, "the observation transitions")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->R, p->R, nm * sizeof(float), fn, "the rewards")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->Z, p->Z, rrz * sizeof(int), fn, "the non-zero belief states")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->B, p->B, rrz * sizeof(float), fn, "the belief points")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->Gamma, per->Gamma, rn * sizeof(float), fn, "Gamma")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->GammaPrime, per->GammaPrime, rn * sizeof(float), fn, "Gamma (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->pi, per->pi, p->r * sizeof(unsigned), fn, "pi")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->piPrime, per->piPrime, p->r * sizeof(unsigned), fn, "pi (prime)")) != NOVA_SUCCESS) return rc;
    DevModel md;
    md.n = p->n; md.ns = p->ns; md.m = p->m; md.z = p->z; md.r = p->r; md.rz = p->rz; md.gamma = p->gamma;
    md.S = ws->S; md.T = ws->T; md.O = ws->O; md.R = ws->R; md.Z = ws->Z; md.B = ws->B;
    return ws->core.build(md, fn);
}

extern "C" int pomdp_perseus_update_cpu(const POMDP *pomdp, POMDPPerseusCPU *per) {
    static const char *fn = "pomdp_perseus_update_cpu";
    if (perseus_shape_invalid(pomdp) || per == nullptr || per->Gamma == nullptr || per->GammaPrime == nullptr ||
            per->pi == nullptr || per->piPrime == nullptr || per->BTilde == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    PerseusCpuWorkspace *ws = perseus_cpu_ws(per);
    if (ws == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized (call pomdp_perseus_initialize_cpu).");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = perseus_cpu_prepare(ws, pomdp, per, fn);
    if (rc != NOVA_SUCCESS) return rc;
    const bool even = (per->currentHorizon % 2u) == 0u;
    unsigned slot = 0;
    float *hostGp = even ? per->GammaPrime : per->Gamma;
    unsigned *hostPiP = even ? per->piPrime : per->pi;
    float *devGp = even ? ws->GammaPrime : ws->Gamma;
    unsigned *devPiP = even ? ws->piPrime : ws->pi;
    if (even)
        rc = ws->core.update(ws->Gamma, ws->pi, ws->GammaPrime, ws->piPrime, per->currentHorizon, per->rGamma,
                             per->rGammaPrime, per->rTilde, per->BTilde, &slot, fn);
    else
        rc = ws->core.update(ws->GammaPrime, ws->piPrime, ws->Gamma, ws->pi, per->currentHorizon, per->rGammaPrime,
                             per->rGamma, per->rTilde, per->BTilde, &slot, fn);
    if (rc != NOVA_SUCCESS && rc != NOVA_CONVERGED) return rc;
    const int rc2 = d2h(hostGp + (size_t)slot * pomdp->n, devGp + (size_t)slot * pomdp->n, pomdp->n * sizeof(float),
                        fn, "Gamma (prime)");
    if (rc2 != NOVA_SUCCESS) return rc2;
    const int rc3 = d2h(hostPiP + slot, devPiP + slot, sizeof(unsigned), fn, "pi (prime)");
    if (rc3 != NOVA_SUCCESS) return rc3;
    return rc;
}

extern "C" int pomdp_perseus_get_policy_cpu(const POMDP *pomdp, POMDPPerseusCPU *per, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_perseus_get_policy_cpu";
    if (pomdp == nullptr || per == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const bool even = (per->currentHorizon % 2u) == 0u;
    const unsigned rows = even ? per->rGamma : per->rGammaPrime;
    if (pomdp_alpha_vectors_initialize(policy, pomdp->n, pomdp->m, rows) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    memcpy(policy->Gamma, even ? per->Gamma : per->GammaPrime, (size_t)rows * pomdp->n * sizeof(float));
    memcpy(policy->pi, even ? per->pi : per->piPrime, rows * sizeof(unsigned));
    return NOVA_SUCCESS;
}

extern "C" int pomdp_perseus_execute_cpu(const POMDP *pomdp, POMDPPerseusCPU *per, POMDPAlphaVectors *policy) {
    static const char *fn = "pomdp_perseus_execute_cpu";
    if (perseus_shape_invalid(pomdp) || pomdp->S == nullptr || pomdp->T == nullptr || pomdp->O == nullptr ||
            pomdp->R == nullptr || pomdp->Z == nullptr || pomdp->B == nullptr || per == nullptr ||
            per->GammaInitial == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int rc = pomdp_perseus_initialize_cpu(pomdp, per);
    if (rc != NOVA_SUCCESS) return rc;
    while (per->currentHorizon < pomdp->horizon) {
        rc = NOVA_SUCCESS;
        while (rc != NOVA_CONVERGED) {
            rc = pomdp_perseus_update_cpu(pomdp, per);
            if (rc != NOVA_CONVERGED && rc != NOVA_SUCCESS) return rc;
        }
    }
    rc = pomdp_perseus_get_policy_cpu(pomdp, per, policy);
    if (rc != NOVA_SUCCESS) return rc;
    return pomdp_perseus_uninitialize_cpu(pomdp, per);
}
