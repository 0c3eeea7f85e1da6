// nova-gb300: MDP value iteration (Bellman sweep) on the GB300.
//
// Replaces mdp_vi_bellman_update_gpu (mdp_vi_gpu.cu:37-87), whose one thread
// per state reads a 512 B row with uncoalesced 4 B loads, and the lifecycle
// functions of mdp_vi_gpu.cu:90-346 / mdp_vi_cpu.cpp:66-223.
//
// Kernel design (memory-bound; HBM roofline):
//   * G lanes per state (G = next power of two >= m); lane a computes Q(s,a)
//     from its own contiguous (s,a) row of S and T with 128-bit loads; the
//     rows of one warp form one contiguous 2 KB span (config n=2^20, m=8,
//     ns=16), so every sector fetched from HBM is used.
//   * V is gathered through the read-only path (4 MiB at n=2^20: L2 resident).
//   * Arithmetic follows mdp_vi_cpu.cpp:36-63 exactly: Q = R(s,a), then for
//     each successor in order Q += (gamma * T) * V[s'] with every product and
//     sum rounded separately; the action scan is the reference's sequential
//     `a == 0 || Q > V'` loop (lowest action on ties, NaN never replaces).
//   * The sweep's Bellman residual max_s |V'(s) - V(s)| is reduced in FP64 in
//     the same pass (one atomic per block).

#include "vi.h"

#include <algorithm>
#include <mutex>
#include <vector>

#include <nova/constants.h>
#include <nova/mdp/mdp.h>
#include <nova/mdp/algorithms/mdp_vi_cpu.h>
#include <nova/mdp/algorithms/mdp_vi_gpu.h>
#include <nova/mdp/policies/mdp_value_function.h>
#include <nova/nova_gb300.h>

using nova::MDP;
using nova::MDPVICPU;
using nova::MDPVIGPU;
using nova::MDPValueFunction;

namespace nova_gb300 {

template <bool VEC>
__device__ __forceinline__ float bellman_q(unsigned s, unsigned a, unsigned m, unsigned ns, float gamma,
                                           const int *__restrict__ S, const float *__restrict__ T,
                                           const float *__restrict__ R, const float *__restrict__ V) {
    float q = __ldg(R + (size_t)s * m + a);
    const size_t row = ((size_t)s * m + a) * ns;
    if (VEC) {
        const int4 *S4 = reinterpret_cast<const int4 *>(S + row);
        const float4 *T4 = reinterpret_cast<const float4 *>(T + row);
        const unsigned nv = ns >> 2;
        for (unsigned c = 0; c < nv; c++) {
            const int4 sv = __ldg(S4 + c);
            const float4 tv = __ldg(T4 + c);
            if (sv.x < 0) break;
            q = fadd(q, fmul(fmul(gamma, tv.x), __ldg(V + sv.x)));
            if (sv.y < 0) break;
            q = fadd(q, fmul(fmul(gamma, tv.y), __ldg(V + sv.y)));
            if (sv.z < 0) break;
            q = fadd(q, fmul(fmul(gamma, tv.z), __ldg(V + sv.z)));
            if (sv.w < 0) break;
            q = fadd(q, fmul(fmul(gamma, tv.w), __ldg(V + sv.w)));
        }
    } else {
        for (unsigned l = 0; l < ns; l++) {
            const int sp = __ldg(S + row + l);
            if (sp < 0) break;
            q = fadd(q, fmul(fmul(gamma, __ldg(T + row + l)), __ldg(V + sp)));
        }
    }
    return q;
}

// One Bellman sweep. G lanes per state, G a power of two in [1, 32], m <= G.
// The grid is a few waves of resident blocks that stride over 256-thread
// tiles, so the residual costs two atomics per block, not per tile.
template <int G, bool VEC>
__global__ void __launch_bounds__(256) bellman_sweep_kernel(unsigned n, unsigned ns, unsigned m, float gamma,
        const int *__restrict__ S, const float *__restrict__ T, const float *__restrict__ R,
        const float *__restrict__ V, float *__restrict__ Vp, unsigned *__restrict__ pi,
        ViDeviceState *st, double tol, int early_exit) {
    if (early_exit && *(volatile unsigned *)&st->converged) return;  // uniform across the grid
    const unsigned long long tiles = ((unsigned long long)n * G + 255ull) / 256ull;
    const unsigned lane = threadIdx.x & 31;
    const unsigned base = lane & ~(unsigned)(G - 1);
    double local = 0.0;
    for (unsigned long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const unsigned long long gid = tile * 256ull + threadIdx.x;
        const unsigned s = (unsigned)(gid / G);
        const unsigned a = (unsigned)(gid % G);
        const bool active_state = s < n;
        float q = 0.0f;
        if (active_state && a < m) q = bellman_q<VEC>(s, a, m, ns, gamma, S, T, R, V);

        // Sequential action scan of mdp_vi_cpu.cpp:55-58 done by the group's lane 0.
        float best = __shfl_sync(0xffffffffu, q, base);
        unsigned besta = 0;
        for (unsigned k = 1; k < m; k++) {
            const float qk = __shfl_sync(0xffffffffu, q, base + k);
            if (qk > best) { best = qk; besta = k; }
        }
        if (active_state && a == 0) {
            Vp[s] = best;
            pi[s] = besta;
            local = fmax(local, fabs((double)best - (double)__ldg(V + s)));
        }
    }
    residual_commit(local, st, gridDim.x, tol, early_exit != 0);
}

// Fallback for m > 32: one thread per state scanning actions in order.
template <bool VEC>
__global__ void __launch_bounds__(256) bellman_sweep_wide_kernel(unsigned n, unsigned ns, unsigned m, float gamma,
        const int *__restrict__ S, const float *__restrict__ T, const float *__restrict__ R,
        const float *__restrict__ V, float *__restrict__ Vp, unsigned *__restrict__ pi,
        ViDeviceState *st, double tol, int early_exit) {
    if (early_exit && *(volatile unsigned *)&st->converged) return;
    const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 0.0;
    if (s < n) {
        float best = 0.0f;
        unsigned besta = 0;
        for (unsigned a = 0; a < m; a++) {
            const float q = bellman_q<VEC>(s, a, m, ns, gamma, S, T, R, V);
            if (a == 0 || q > best) { best = q; besta = a; }
        }
        Vp[s] = best;
        pi[s] = besta;
        local = fabs((double)best - (double)__ldg(V + s));
    }
    residual_commit(local, st, gridDim.x, tol, early_exit != 0);
}

// Resident 256-thread blocks per SM times the SM count of the current device.
static unsigned resident_blocks() {
    static std::mutex mu;
    static unsigned cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1216u;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (cache[dev] == 0) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            sms = 152;
        }
        cache[dev] = (unsigned)sms * 8u;
    }
    return cache[dev];
}

template <int G>
static void launch_group(unsigned n, unsigned ns, unsigned m, float gamma, const int *S, const float *T,
                         const float *R, const float *V, float *Vp, unsigned *pi, ViDeviceState *st,
                         double tol, int early_exit, bool vec, cudaStream_t stream) {
    const unsigned long long tiles = ((unsigned long long)n * G + 255ull) / 256ull;
    const unsigned blocks = (unsigned)std::min<unsigned long long>(tiles, resident_blocks());
    if (vec)
        bellman_sweep_kernel<G, true><<<blocks, 256, 0, stream>>>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit);
    else
        bellman_sweep_kernel<G, false><<<blocks, 256, 0, stream>>>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit);
}

// Launch one sweep V -> Vp. Returns NOVA_SUCCESS or a launch error.
static int launch_sweep(const MDP *mdp, const int *S, const float *T, const float *R, const float *V, float *Vp,
                        unsigned *pi, ViDeviceState *st, double tol, int early_exit, cudaStream_t stream,
                        ViTilePlan *plan, const char *fn) {
    if (plan != nullptr) {
        // The plan is built at the solver's first sweep from the model as it
        // is then; the tiled sweep needs V and R 16-byte aligned for its bulk
        // copies.
        int rc = vi_plan_build(plan, mdp, S, T, stream, fn);
        if (rc != NOVA_SUCCESS) return rc;
        if (plan->status == ViTilePlan::kTiled && ((uintptr_t)V % 16u) == 0u && ((uintptr_t)R % 16u) == 0u)
            return vi_tiled_sweep(plan, mdp, R, V, Vp, pi, st, tol, early_exit, stream, fn);
    }
    const unsigned n = mdp->n, ns = mdp->ns, m = mdp->m;
    const float gamma = mdp->gamma;
    const bool vec = (ns % 4u) == 0u && ((uintptr_t)S % 16u) == 0u && ((uintptr_t)T % 16u) == 0u;
    if (m > 32) {
        const unsigned blocks = ceil_div(n, 256);
        if (vec)
            bellman_sweep_wide_kernel<true><<<blocks, 256, 0, stream>>>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit);
        else
            bellman_sweep_wide_kernel<false><<<blocks, 256, 0, stream>>>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit);
    } else if (m > 16) {
        launch_group<32>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    } else if (m > 8) {
        launch_group<16>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    } else if (m > 4) {
        launch_group<8>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    } else if (m > 2) {
        launch_group<4>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    } else if (m > 1) {
        launch_group<2>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    } else {
        launch_group<1>(n, ns, m, gamma, S, T, R, V, Vp, pi, st, tol, early_exit, vec, stream);
    }
    return check_launch(fn, "Bellman update");
}

// ---------------------------------------------------------------------------
// Workspaces
// ---------------------------------------------------------------------------

// Device-side solver state of MDPVIGPU beyond its ABI fields.
struct ViGpuWorkspace : Workspace {
    float *d_V = nullptr, *d_VPrime = nullptr;
    unsigned *d_pi = nullptr;
    ViDeviceState *st = nullptr;
    ViTilePlan plan;
    ~ViGpuWorkspace() override {
        cudaFree(d_V); cudaFree(d_VPrime); cudaFree(d_pi); cudaFree(st);
    }
};

// Host-buffer solver (MDPVICPU): device copies of the model and of V, V', pi.
struct ViCpuWorkspace : Workspace {
    int *S = nullptr;
    float *T = nullptr, *R = nullptr;
    float *V = nullptr, *VPrime = nullptr;
    unsigned *pi = nullptr;
    ViDeviceState *st = nullptr;
    float *hostV = nullptr, *hostVPrime = nullptr;   // the arrays this library gave the struct
    unsigned *hostPi = nullptr;
    ViTilePlan plan;
    ~ViCpuWorkspace() override {
        cudaFree(S); cudaFree(T); cudaFree(R); cudaFree(V); cudaFree(VPrime); cudaFree(pi); cudaFree(st);
    }
};

static int alloc_state(ViDeviceState **st, const char *fn) {
    int rc = dev_alloc(st, 1, fn, "the convergence state");
    if (rc != NOVA_SUCCESS) return rc;
    if (cudaMemset(*st, 0, sizeof(ViDeviceState)) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to clear the convergence state.");
        return NOVA_ERROR_MEMCPY_TO_DEVICE;
    }
    return NOVA_SUCCESS;
}

}  // namespace nova_gb300

using namespace nova_gb300;

// ===========================================================================
// Device-buffer value iteration (mdp_vi_gpu.cu)
// ===========================================================================

extern "C" int mdp_vi_uninitialize_gpu(const MDP *mdp, MDPVIGPU *vi) {
    if (mdp == nullptr || vi == nullptr) {
        NOVA_ERR("mdp_vi_uninitialize_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    vi->currentHorizon = 0;
    int result = NOVA_SUCCESS;
    std::lock_guard<std::mutex> lock(registry_mutex());
    auto *ws = find_workspace<ViGpuWorkspace>(vi);
    if (ws != nullptr) {
        // Free only what this library allocated; fields the caller replaced
        // are left alone.
        if (vi->d_V == ws->d_V) vi->d_V = nullptr;
        if (vi->d_VPrime == ws->d_VPrime) vi->d_VPrime = nullptr;
        if (vi->d_pi == ws->d_pi) vi->d_pi = nullptr;
        cudaDeviceSynchronize();
        registry().erase(vi);
    }
    // Pointers not owned by a workspace are freed as the reference does
    // (mdp_vi_gpu.cu:224-266).
    if (vi->d_V != nullptr && dev_free(vi->d_V, "mdp_vi_uninitialize_gpu", "the value function") != NOVA_SUCCESS)
        result = NOVA_ERROR_DEVICE_FREE;
    vi->d_V = nullptr;
    if (vi->d_VPrime != nullptr &&
            dev_free(vi->d_VPrime, "mdp_vi_uninitialize_gpu", "the value function (prime)") != NOVA_SUCCESS)
        result = NOVA_ERROR_DEVICE_FREE;
    vi->d_VPrime = nullptr;
    if (vi->d_pi != nullptr && dev_free(vi->d_pi, "mdp_vi_uninitialize_gpu", "the policy (pi)") != NOVA_SUCCESS)
        result = NOVA_ERROR_DEVICE_FREE;
    vi->d_pi = nullptr;
    return result;
}

extern "C" int mdp_vi_initialize_gpu(const MDP *mdp, MDPVIGPU *vi) {
    static const char *fn = "mdp_vi_initialize_gpu";
    if (mdp == nullptr || mdp->n == 0 || vi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    vi->currentHorizon = 0;
    {
        // Idempotent: release what an earlier initialize on this struct made.
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *old = find_workspace<ViGpuWorkspace>(vi);
        if (old != nullptr) {
            if (vi->d_V == old->d_V) vi->d_V = nullptr;
            if (vi->d_VPrime == old->d_VPrime) vi->d_VPrime = nullptr;
            if (vi->d_pi == old->d_pi) vi->d_pi = nullptr;
            registry().erase(vi);
        }
    }
    const unsigned n = mdp->n;
    std::unique_ptr<ViGpuWorkspace> ws(new ViGpuWorkspace());
    int rc;
    if ((rc = dev_alloc(&ws->d_V, n, fn, "the value function")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_VPrime, n, fn, "the value function (prime)")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&ws->d_pi, n, fn, "the policy (pi)")) != NOVA_SUCCESS) return rc;
    if ((rc = alloc_state(&ws->st, fn)) != NOVA_SUCCESS) return rc;
    // VInitial == nullptr means V = 0 (mdp_vi_gpu.cu:100-106).
    std::vector<float> zeros;
    const float *init = vi->VInitial;
    if (init == nullptr) {
        zeros.assign(n, 0.0f);
        init = zeros.data();
    }
    if ((rc = h2d(ws->d_V, init, n * sizeof(float), fn, "the value function")) != NOVA_SUCCESS) return rc;
    if ((rc = h2d(ws->d_VPrime, init, n * sizeof(float), fn, "the value function (prime)")) != NOVA_SUCCESS) return rc;
    if (cudaMemset(ws->d_pi, 0, n * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to copy memory from host to device for pi.");
        return NOVA_ERROR_MEMCPY_TO_DEVICE;
    }
    vi->d_V = ws->d_V;
    vi->d_VPrime = ws->d_VPrime;
    vi->d_pi = ws->d_pi;
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[vi] = std::move(ws);
    return NOVA_SUCCESS;
}

static int vi_gpu_sweep(const MDP *mdp, MDPVIGPU *vi, double tol, int early_exit, bool sync, const char *fn) {
    ViDeviceState *st = nullptr;
    ViTilePlan *plan = nullptr;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *ws = find_workspace<ViGpuWorkspace>(vi);
        if (ws != nullptr) {
            st = ws->st;
            plan = &ws->plan;
        }
    }
    if (st == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const bool even = (vi->currentHorizon % 2u) == 0u;
    const float *src = even ? vi->d_V : vi->d_VPrime;
    float *dst = even ? vi->d_VPrime : vi->d_V;
    int rc = launch_sweep(mdp, mdp->d_S, mdp->d_T, mdp->d_R, src, dst, vi->d_pi, st, tol, early_exit, 0, plan, fn);
    if (rc != NOVA_SUCCESS) return rc;
    if (sync) {
        rc = sync_device(fn);
        if (rc == NOVA_SUCCESS) rc = vi_state_error(st, fn);
        if (rc != NOVA_SUCCESS) return rc;
    }
    vi->currentHorizon++;
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_update_gpu(const MDP *mdp, MDPVIGPU *vi) {
    static const char *fn = "mdp_vi_update_gpu";
    if (mdp == nullptr || vi == nullptr || mdp->d_S == nullptr || mdp->d_T == nullptr || mdp->d_R == nullptr ||
            vi->d_V == nullptr || vi->d_VPrime == nullptr || vi->d_pi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    return vi_gpu_sweep(mdp, vi, 0.0, 0, true, fn);
}

extern "C" int mdp_vi_get_policy_gpu(const MDP *mdp, MDPVIGPU *vi, MDPValueFunction *policy) {
    static const char *fn = "mdp_vi_get_policy_gpu";
    if (mdp == nullptr || vi == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (mdp_value_function_initialize(policy, mdp->n, mdp->m, 0) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    const float *src = (vi->currentHorizon % 2u == 0u) ? vi->d_V : vi->d_VPrime;
    int rc = d2h(policy->V, src, mdp->n * sizeof(float), fn, "the value function");
    if (rc != NOVA_SUCCESS) return rc;
    return d2h(policy->pi, vi->d_pi, mdp->n * sizeof(unsigned), fn, "the policy (pi)");
}

static int vi_validate_execute(const MDP *mdp, const void *vi, const void *policy, bool device, const char *fn) {
    // Validation list of mdp_vi_gpu.cu:166-172 / mdp_vi_cpu.cpp:104-110.
    if (mdp == nullptr || mdp->n == 0 || mdp->ns == 0 || mdp->m == 0 ||
            mdp->S == nullptr || mdp->T == nullptr || mdp->R == nullptr ||
            mdp->gamma < 0.0f || mdp->gamma > 1.0f || mdp->horizon < 1 ||
            vi == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (device && (mdp->d_S == nullptr || mdp->d_T == nullptr || mdp->d_R == nullptr)) {
        NOVA_ERR(fn, "Invalid arguments: the MDP has no device copy (call mdp_initialize_gpu).");
        return NOVA_ERROR_INVALID_DATA;
    }
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_execute_gpu(const MDP *mdp, MDPVIGPU *vi, MDPValueFunction *policy) {
    static const char *fn = "mdp_vi_execute_gpu";
    int rc = vi_validate_execute(mdp, vi, policy, true, fn);
    if (rc != NOVA_SUCCESS) return rc;
    if (vi->numThreads % 32 != 0) {
        NOVA_ERR(fn, "Invalid number of threads.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    rc = mdp_vi_initialize_gpu(mdp, vi);
    if (rc != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Failed to initialize GPU variables.");
        return rc;
    }
    // Sweeps are queued back to back on the stream; one synchronisation at
    // the end replaces the reference's per-sweep cudaDeviceSynchronize.
    while (vi->currentHorizon < mdp->horizon) {
        rc = vi_gpu_sweep(mdp, vi, 0.0, 0, false, fn);
        if (rc != NOVA_SUCCESS) {
            mdp_vi_uninitialize_gpu(mdp, vi);
            return rc;
        }
    }
    rc = sync_device(fn);
    if (rc == NOVA_SUCCESS) {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *ws = find_workspace<ViGpuWorkspace>(vi);
        if (ws != nullptr) rc = vi_state_error(ws->st, fn);
    }
    if (rc == NOVA_SUCCESS) rc = mdp_vi_get_policy_gpu(mdp, vi, policy);
    if (rc != NOVA_SUCCESS) {
        mdp_vi_uninitialize_gpu(mdp, vi);
        return rc;
    }
    return mdp_vi_uninitialize_gpu(mdp, vi);
}

extern "C" int mdp_vi_residual_gpu(const MDP *mdp, const MDPVIGPU *vi, double *residual) {
    static const char *fn = "mdp_vi_residual_gpu";
    if (mdp == nullptr || vi == nullptr || residual == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    ViDeviceState *st = nullptr;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *ws = find_workspace<ViGpuWorkspace>(vi);
        if (ws != nullptr) st = ws->st;
    }
    if (st == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized.");
        return NOVA_ERROR_INVALID_DATA;
    }
    ViDeviceState h;
    int rc = d2h(&h, st, sizeof(h), fn, "the convergence state");
    if (rc != NOVA_SUCCESS) return rc;
    *residual = h.last_resid;
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_execute_until_converged_gpu(const MDP *mdp, MDPVIGPU *vi, MDPValueFunction *policy,
        double tol, unsigned int maxSweeps, unsigned int *sweeps, double *residual) {
    static const char *fn = "mdp_vi_execute_until_converged_gpu";
    int rc = vi_validate_execute(mdp, vi, policy, true, fn);
    if (rc != NOVA_SUCCESS) return rc;
    if (vi->numThreads % 32 != 0) {
        NOVA_ERR(fn, "Invalid number of threads.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    if (!(tol >= 0.0) || maxSweeps == 0) {
        NOVA_ERR(fn, "Invalid arguments: tol must be >= 0 and maxSweeps > 0.");
        return NOVA_ERROR_INVALID_DATA;
    }
    rc = mdp_vi_initialize_gpu(mdp, vi);
    if (rc != NOVA_SUCCESS) return rc;
    ViDeviceState *st = nullptr;
    ViTilePlan *plan = nullptr;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *ws = find_workspace<ViGpuWorkspace>(vi);
        st = ws->st;
        plan = &ws->plan;
    }
    // Sweeps are queued in batches; a sweep launched after convergence
    // returns at once, so the device state ends at the first converged sweep.
    const unsigned kBatch = 32;
    unsigned launched = 0;
    ViDeviceState h;
    memset(&h, 0, sizeof(h));
    while (launched < maxSweeps) {
        const unsigned b = (maxSweeps - launched) < kBatch ? (maxSweeps - launched) : kBatch;
        for (unsigned k = 0; k < b; k++) {
            const bool even = (launched % 2u) == 0u;
            const float *src = even ? vi->d_V : vi->d_VPrime;
            float *dst = even ? vi->d_VPrime : vi->d_V;
            rc = launch_sweep(mdp, mdp->d_S, mdp->d_T, mdp->d_R, src, dst, vi->d_pi, st, tol, 1, 0, plan, fn);
            if (rc != NOVA_SUCCESS) { mdp_vi_uninitialize_gpu(mdp, vi); return rc; }
            launched++;
        }
        rc = d2h(&h, st, sizeof(h), fn, "the convergence state");
        if (rc == NOVA_SUCCESS) rc = vi_state_error(st, fn);
        if (rc != NOVA_SUCCESS) { mdp_vi_uninitialize_gpu(mdp, vi); return rc; }
        if (h.converged) break;
    }
    vi->currentHorizon = h.sweeps_done;
    if (sweeps) *sweeps = h.sweeps_done;
    if (residual) *residual = h.last_resid;
    rc = mdp_vi_get_policy_gpu(mdp, vi, policy);
    if (rc != NOVA_SUCCESS) { mdp_vi_uninitialize_gpu(mdp, vi); return rc; }
    return mdp_vi_uninitialize_gpu(mdp, vi);
}

// ===========================================================================
// Host-buffer value iteration (mdp_vi_cpu.cpp): same kernels, host arrays
// ===========================================================================

extern "C" int mdp_vi_uninitialize_cpu(const MDP *mdp, MDPVICPU *vi) {
    if (mdp == nullptr || vi == nullptr) {
        NOVA_ERR("mdp_vi_uninitialize_cpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    vi->currentHorizon = 0;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        registry().erase(vi);
    }
    // Host arrays are new[] allocations, freed as mdp_vi_cpu.cpp:165-178.
    delete[] vi->V; vi->V = nullptr;
    delete[] vi->VPrime; vi->VPrime = nullptr;
    delete[] vi->pi; vi->pi = nullptr;
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_initialize_cpu(const MDP *mdp, MDPVICPU *vi) {
    static const char *fn = "mdp_vi_initialize_cpu";
    if (mdp == nullptr || mdp->n == 0 || vi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned n = mdp->n;
    vi->currentHorizon = 0;
    {
        // Idempotent on this struct: drop arrays an earlier call made.
        std::lock_guard<std::mutex> lock(registry_mutex());
        auto *old = find_workspace<ViCpuWorkspace>(vi);
        if (old != nullptr) {
            if (vi->V == old->hostV) { delete[] vi->V; vi->V = nullptr; }
            if (vi->VPrime == old->hostVPrime) { delete[] vi->VPrime; vi->VPrime = nullptr; }
            if (vi->pi == old->hostPi) { delete[] vi->pi; vi->pi = nullptr; }
            registry().erase(vi);
        }
    }
    vi->V = new float[n];
    vi->VPrime = new float[n];
    vi->pi = new unsigned int[n];
    for (unsigned i = 0; i < n; i++) {
        const float v = vi->VInitial != nullptr ? vi->VInitial[i] : 0.0f;
        vi->V[i] = v;
        vi->VPrime[i] = v;
        vi->pi[i] = 0;
    }
    // The model is read here: later updates use this snapshot of S, T, R.
    std::unique_ptr<ViCpuWorkspace> ws(new ViCpuWorkspace());
    ws->hostV = vi->V; ws->hostVPrime = vi->VPrime; ws->hostPi = vi->pi;
    if (mdp->S != nullptr && mdp->T != nullptr && mdp->R != nullptr && mdp->ns > 0 && mdp->m > 0) {
        const size_t nms = (size_t)n * mdp->m * mdp->ns;
        int rc;
        if ((rc = dev_alloc(&ws->S, nms, fn, "the successor states")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&ws->T, nms, fn, "the state transitions")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&ws->R, (size_t)n * mdp->m, fn, "the rewards")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&ws->V, n, fn, "the value function")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&ws->VPrime, n, fn, "the value function (prime)")) != NOVA_SUCCESS) return rc;
        if ((rc = dev_alloc(&ws->pi, n, fn, "the policy (pi)")) != NOVA_SUCCESS) return rc;
        if ((rc = alloc_state(&ws->st, fn)) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(ws->S, mdp->S, nms * sizeof(int), fn, "the successor states")) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(ws->T, mdp->T, nms * sizeof(float), fn, "the state transitions")) != NOVA_SUCCESS) return rc;
        if ((rc = h2d(ws->R, mdp->R, (size_t)n * mdp->m * sizeof(float), fn, "the rewards")) != NOVA_SUCCESS) return rc;
    }
    std::lock_guard<std::mutex> lock(registry_mutex());
    registry()[vi] = std::move(ws);
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_update_cpu(const MDP *mdp, MDPVICPU *vi) {
    static const char *fn = "mdp_vi_update_cpu";
    if (mdp == nullptr || vi == nullptr || vi->V == nullptr || vi->VPrime == nullptr || vi->pi == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    ViCpuWorkspace *ws;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        ws = find_workspace<ViCpuWorkspace>(vi);
    }
    if (ws == nullptr || ws->S == nullptr) {
        NOVA_ERR(fn, "The solver is not initialized with a complete MDP.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned n = mdp->n;
    const bool even = (vi->currentHorizon % 2u) == 0u;
    float *hsrc = even ? vi->V : vi->VPrime;
    float *hdst = even ? vi->VPrime : vi->V;
    // Host arrays are the source of truth between calls (callers may edit them).
    int rc = h2d(ws->V, hsrc, n * sizeof(float), fn, "the value function");
    if (rc != NOVA_SUCCESS) return rc;
    rc = launch_sweep(mdp, ws->S, ws->T, ws->R, ws->V, ws->VPrime, ws->pi, ws->st, 0.0, 0, 0, &ws->plan, fn);
    if (rc != NOVA_SUCCESS) return rc;
    rc = d2h(hdst, ws->VPrime, n * sizeof(float), fn, "the value function (prime)");
    if (rc == NOVA_SUCCESS) rc = vi_state_error(ws->st, fn);
    if (rc != NOVA_SUCCESS) return rc;
    rc = d2h(vi->pi, ws->pi, n * sizeof(unsigned), fn, "the policy (pi)");
    if (rc != NOVA_SUCCESS) return rc;
    vi->currentHorizon++;
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_get_policy_cpu(const MDP *mdp, MDPVICPU *vi, MDPValueFunction *policy) {
    static const char *fn = "mdp_vi_get_policy_cpu";
    if (mdp == nullptr || vi == nullptr || policy == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (mdp_value_function_initialize(policy, mdp->n, mdp->m, 0) != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Could not create the policy.");
        return NOVA_ERROR_POLICY_CREATION;
    }
    const float *src = (vi->currentHorizon % 2u == 0u) ? vi->V : vi->VPrime;
    memcpy(policy->V, src, mdp->n * sizeof(float));
    memcpy(policy->pi, vi->pi, mdp->n * sizeof(unsigned));
    return NOVA_SUCCESS;
}

extern "C" int mdp_vi_execute_cpu(const MDP *mdp, MDPVICPU *vi, MDPValueFunction *policy) {
    static const char *fn = "mdp_vi_execute_cpu";
    int rc = vi_validate_execute(mdp, vi, policy, false, fn);
    if (rc != NOVA_SUCCESS) return rc;
    rc = mdp_vi_initialize_cpu(mdp, vi);
    if (rc != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Failed to initialize the CPU variables.");
        return rc;
    }
    ViCpuWorkspace *ws;
    {
        std::lock_guard<std::mutex> lock(registry_mutex());
        ws = find_workspace<ViCpuWorkspace>(vi);
    }
    const unsigned n = mdp->n;
    // The whole solve stays on the device; V, V' and pi are copied back once.
    rc = h2d(ws->V, vi->V, n * sizeof(float), fn, "the value function");
    if (rc == NOVA_SUCCESS) rc = h2d(ws->VPrime, vi->VPrime, n * sizeof(float), fn, "the value function (prime)");
    while (rc == NOVA_SUCCESS && vi->currentHorizon < mdp->horizon) {
        const bool even = (vi->currentHorizon % 2u) == 0u;
        rc = launch_sweep(mdp, ws->S, ws->T, ws->R, even ? ws->V : ws->VPrime, even ? ws->VPrime : ws->V, ws->pi,
                          ws->st, 0.0, 0, 0, &ws->plan, fn);
        if (rc == NOVA_SUCCESS) vi->currentHorizon++;
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    if (rc == NOVA_SUCCESS) rc = vi_state_error(ws->st, fn);
    if (rc == NOVA_SUCCESS) rc = d2h(vi->V, ws->V, n * sizeof(float), fn, "the value function");
    if (rc == NOVA_SUCCESS) rc = d2h(vi->VPrime, ws->VPrime, n * sizeof(float), fn, "the value function (prime)");
    if (rc == NOVA_SUCCESS) rc = d2h(vi->pi, ws->pi, n * sizeof(unsigned), fn, "the policy (pi)");
    if (rc == NOVA_SUCCESS) rc = mdp_vi_get_policy_cpu(mdp, vi, policy);
    if (rc != NOVA_SUCCESS) {
        NOVA_ERR(fn, "Failed to perform Bellman update on the GPU.");
        mdp_vi_uninitialize_cpu(mdp, vi);
        return rc;
    }
    return mdp_vi_uninitialize_cpu(mdp, vi);
}

extern "C" int mdp_vi_tiling_status_gpu(const void *vi, unsigned int *status) {
    if (status == nullptr) {
        NOVA_ERR("mdp_vi_tiling_status_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (vi == nullptr) {
        *status = vi_last_plan_status();
        return NOVA_SUCCESS;
    }
    std::lock_guard<std::mutex> lock(registry_mutex());
    if (auto *g = find_workspace<ViGpuWorkspace>(vi)) {
        *status = g->plan.status;
        return NOVA_SUCCESS;
    }
    if (auto *c = find_workspace<ViCpuWorkspace>(vi)) {
        *status = c->plan.status;
        return NOVA_SUCCESS;
    }
    NOVA_ERR("mdp_vi_tiling_status_gpu", "The solver is not initialized.");
    return NOVA_ERROR_INVALID_DATA;
}
