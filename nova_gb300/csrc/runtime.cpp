// nova-gb300 host runtime: CUDA wrappers with NOVA_* error mapping, fault
// injection, the workspace registry, host model allocation (POMDP / MDP),
// device model upload, and the policy containers.
//
// Model and policy entry points keep the reference's semantics and error
// codes; each cites the reference function it replaces.

#include "common.h"

#include <cmath>
#include <atomic>

#include <nova/constants.h>
#include <nova/pomdp/pomdp.h>
#include <nova/mdp/mdp.h>
#include <nova/pomdp/utilities/pomdp_model_cpu.h>
#include <nova/pomdp/utilities/pomdp_model_gpu.h>
#include <nova/mdp/utilities/mdp_model_cpu.h>
#include <nova/mdp/utilities/mdp_model_gpu.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>
#include <nova/mdp/policies/mdp_value_function.h>
#include <nova/nova_gb300.h>

namespace nova_gb300 {

// ---------------------------------------------------------------------------
// Fault injection and CUDA wrappers
// ---------------------------------------------------------------------------
static std::atomic<unsigned> g_fault_kind{0};
static std::atomic<unsigned> g_fault_countdown{0};

bool fault_fires(FaultKind kind) {
    if (g_fault_kind.load() != (unsigned)kind) return false;
    unsigned left = g_fault_countdown.load();
    if (left == 0) return false;
    if (left == 1) {
        g_fault_countdown.store(0);
        g_fault_kind.store(0);
        return true;
    }
    g_fault_countdown.store(left - 1);
    return false;
}

int dev_malloc(void **p, size_t bytes, const char *fn, const char *what) {
    *p = nullptr;
    if (fault_fires(kFaultMalloc) || cudaMalloc(p, bytes == 0 ? 4 : bytes) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to allocate device-side memory for %s.", what);
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_DEVICE_MALLOC;
    }
    return NOVA_SUCCESS;
}

int dev_free(void *p, const char *fn, const char *what) {
    if (p == nullptr) return NOVA_SUCCESS;
    if (cudaFree(p) != cudaSuccess) {
        cudaGetLastError();
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to free device-side memory for %s.", what);
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_DEVICE_FREE;
    }
    return NOVA_SUCCESS;
}

int h2d(void *dst, const void *src, size_t bytes, const char *fn, const char *what) {
    if (bytes == 0) return NOVA_SUCCESS;
    if (fault_fires(kFaultH2D) || cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to copy memory from host to device for %s.", what);
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_MEMCPY_TO_DEVICE;
    }
    return NOVA_SUCCESS;
}

int d2h(void *dst, const void *src, size_t bytes, const char *fn, const char *what) {
    if (bytes == 0) return NOVA_SUCCESS;
    if (fault_fires(kFaultD2H) || cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to copy memory from device to host for %s.", what);
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    return NOVA_SUCCESS;
}

static std::atomic<unsigned long long> g_launches{0};

unsigned long long launch_count() { return g_launches.load(); }

void add_launches(long long delta) { g_launches.fetch_add((unsigned long long)delta); }

int check_launch(const char *fn, const char *what) {
    g_launches.fetch_add(1);
    cudaError_t e = cudaGetLastError();
    if (fault_fires(kFaultLaunch) || e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to execute the '%s' kernel (%s).", what,
                 e == cudaSuccess ? "injected" : cudaGetErrorString(e));
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    return NOVA_SUCCESS;
}

int sync_device(const char *fn) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "Failed to synchronize the device (%s).", cudaGetErrorString(e));
        NOVA_ERR(fn, msg);
        return NOVA_ERROR_DEVICE_SYNCHRONIZE;
    }
    return NOVA_SUCCESS;
}

std::mutex &registry_mutex() {
    static std::mutex m;
    return m;
}

std::unordered_map<const void *, std::unique_ptr<Workspace>> &registry() {
    static std::unordered_map<const void *, std::unique_ptr<Workspace>> r;
    return r;
}

// Upload one host array into a fresh device allocation, in the reference's
// per-array form (pomdp_model_gpu.cu:78-101): allocate, then copy.
template <typename T>
static int upload_array(T **dptr, const T *host, size_t count, const char *fn, const char *what) {
    int rc = dev_alloc(dptr, count, fn, what);
    if (rc != NOVA_SUCCESS) return rc;
    return h2d(*dptr, host, count * sizeof(T), fn, what);
}

template <typename T>
static int free_array(T **dptr, const char *fn, const char *what) {
    int rc = NOVA_SUCCESS;
    if (*dptr != nullptr) rc = dev_free(*dptr, fn, what);
    if (rc == NOVA_SUCCESS) *dptr = nullptr;
    return rc;
}

}  // namespace nova_gb300

using namespace nova_gb300;
using nova::POMDP;
using nova::MDP;
using nova::POMDPAlphaVectors;
using nova::MDPValueFunction;

// ===========================================================================
// Host POMDP model (pomdp_model_cpu.cpp)
// ===========================================================================

extern "C" int pomdp_initialize_cpu(POMDP *pomdp, unsigned int n, unsigned int ns, unsigned int m,
        unsigned int z, unsigned int r, unsigned int rz, float gamma, unsigned int horizon) {
    // Validation list of pomdp_model_cpu.cpp:37-43.
    if (pomdp == nullptr || pomdp->S != nullptr || pomdp->T != nullptr || pomdp->O != nullptr ||
            pomdp->R != nullptr || pomdp->Z != nullptr || pomdp->B != nullptr ||
            n == 0 || ns == 0 || n < ns || m == 0 || z == 0 || r == 0 || rz == 0 ||
            gamma < 0.0f || gamma > 1.0f || horizon == 0) {
        NOVA_ERR("pomdp_initialize_cpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pomdp->n = n; pomdp->ns = ns; pomdp->m = m; pomdp->z = z; pomdp->r = r; pomdp->rz = rz;
    pomdp->gamma = gamma; pomdp->horizon = horizon;

    const size_t nms = (size_t)n * m * ns;
    pomdp->S = new int[nms];
    pomdp->T = new float[nms];
    for (size_t i = 0; i < nms; i++) { pomdp->S[i] = -1; pomdp->T[i] = 0.0f; }
    pomdp->O = new float[(size_t)m * n * z]();
    pomdp->R = new float[(size_t)n * m]();
    // The reference fills Z with 0 (not -1) here (pomdp_model_cpu.cpp:70-74).
    pomdp->Z = new int[(size_t)r * rz]();
    pomdp->B = new float[(size_t)r * rz]();

    pomdp->d_S = nullptr; pomdp->d_T = nullptr; pomdp->d_O = nullptr;
    pomdp->d_R = nullptr; pomdp->d_Z = nullptr; pomdp->d_B = nullptr;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_belief_update_cpu(const POMDP *pomdp, const float *b, unsigned int a,
        unsigned int o, float *&bp) {
    // Semantics of pomdp_model_cpu.cpp:89-137: forward projection through
    // T(.,a,.), weighting by O(a,.,o), normalisation. Summation order is the
    // reference's (states ascending, successors ascending).
    if (pomdp == nullptr || pomdp->n == 0 || pomdp->ns == 0 || pomdp->m == 0 || pomdp->z == 0 ||
            pomdp->S == nullptr || pomdp->T == nullptr || pomdp->O == nullptr || pomdp->R == nullptr ||
            bp != nullptr || b == nullptr || a >= pomdp->m || o >= pomdp->z) {
        NOVA_ERR("pomdp_belief_update_cpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned n = pomdp->n, m = pomdp->m, ns = pomdp->ns, z = pomdp->z;
    float *out = new float[n]();
    for (unsigned s = 0; s < n; s++) {
        for (unsigned l = 0; l < ns; l++) {
            int sp = pomdp->S[(size_t)s * m * ns + a * ns + l];
            if (sp < 0) break;
            out[sp] += pomdp->T[(size_t)s * m * ns + a * ns + l] * b[s];
        }
    }
    float norm = 0.0f;
    for (unsigned sp = 0; sp < n; sp++) {
        out[sp] *= pomdp->O[(size_t)a * n * z + (size_t)sp * z + o];
        norm += out[sp];
    }
    bp = out;
    if (std::fabs(norm) < NOVA_FLT_ERR_TOL) {
        NOVA_ERR("pomdp_belief_update_cpu",
                 "Computed belief is invalid. The observation is impossible given the belief and action.");
        return NOVA_WARNING_INVALID_BELIEF;
    }
    for (unsigned sp = 0; sp < n; sp++) out[sp] /= norm;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_add_new_raw_beliefs_cpu(POMDP *pomdp, unsigned int numBeliefsToAdd, float *Bnew) {
    // Semantics of pomdp_model_cpu.cpp:157-227 (which lacks its return
    // statement; this one returns NOVA_SUCCESS).
    if (pomdp == nullptr || pomdp->n == 0 || pomdp->ns == 0 || pomdp->m == 0 || pomdp->z == 0 ||
            numBeliefsToAdd == 0 || Bnew == nullptr) {
        NOVA_ERR("pomdp_add_new_beliefs_raw_cpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const unsigned n = pomdp->n;
    const unsigned rOld = pomdp->r, rzOld = pomdp->rz;
    unsigned rzNew = rzOld;
    for (unsigned i = 0; i < numBeliefsToAdd; i++) {
        unsigned nz = 0;
        for (unsigned s = 0; s < n; s++) nz += Bnew[(size_t)i * n + s] > 0.0f ? 1u : 0u;
        if (nz > rzNew) rzNew = nz;
    }
    const unsigned rNew = rOld + numBeliefsToAdd;
    int *Zf = new int[(size_t)rNew * rzNew];
    float *Bf = new float[(size_t)rNew * rzNew];
    for (unsigned i = 0; i < rOld; i++) {
        for (unsigned k = 0; k < rzNew; k++) {
            Zf[(size_t)i * rzNew + k] = k < rzOld ? pomdp->Z[(size_t)i * rzOld + k] : -1;
            Bf[(size_t)i * rzNew + k] = k < rzOld ? pomdp->B[(size_t)i * rzOld + k] : 0.0f;
        }
    }
    for (unsigned i = 0; i < numBeliefsToAdd; i++) {
        unsigned k = 0;
        for (unsigned s = 0; s < n; s++) {
            float v = Bnew[(size_t)i * n + s];
            if (v > 0.0f) {
                Zf[(size_t)(rOld + i) * rzNew + k] = (int)s;
                Bf[(size_t)(rOld + i) * rzNew + k] = v;
                k++;
            }
        }
        for (; k < rzNew; k++) {
            Zf[(size_t)(rOld + i) * rzNew + k] = -1;
            Bf[(size_t)(rOld + i) * rzNew + k] = 0.0f;
        }
    }
    delete[] pomdp->Z;
    delete[] pomdp->B;
    pomdp->r = rNew;
    pomdp->rz = rzNew;
    pomdp->Z = Zf;
    pomdp->B = Bf;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_uninitialize_cpu(POMDP *pomdp) {
    if (pomdp == nullptr) {
        NOVA_ERR("pomdp_uninitialize_cpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    pomdp->n = 0; pomdp->ns = 0; pomdp->m = 0; pomdp->z = 0; pomdp->r = 0; pomdp->rz = 0;
    pomdp->gamma = 0.0f; pomdp->horizon = 0;
    delete[] pomdp->S; pomdp->S = nullptr;
    delete[] pomdp->T; pomdp->T = nullptr;
    delete[] pomdp->O; pomdp->O = nullptr;
    delete[] pomdp->R; pomdp->R = nullptr;
    delete[] pomdp->Z; pomdp->Z = nullptr;
    delete[] pomdp->B; pomdp->B = nullptr;
    return NOVA_SUCCESS;
}

// ===========================================================================
// Device POMDP model (pomdp_model_gpu.cu)
// ===========================================================================

#define POMDP_ARRAY_PAIR(NAME, FIELD, DFIELD, TYPE, COUNT, CHECK, WHAT)                          \
    extern "C" int pomdp_initialize_##NAME##_gpu(POMDP *pomdp) {                               \
        if (pomdp == nullptr || (CHECK) || pomdp->FIELD == nullptr) {                          \
            NOVA_ERR("pomdp_initialize_" #NAME "_gpu", "Invalid input.");                     \
            return NOVA_ERROR_INVALID_DATA;                                                    \
        }                                                                                      \
        return upload_array<TYPE>(&pomdp->DFIELD, pomdp->FIELD, (COUNT),                       \
                                  "pomdp_initialize_" #NAME "_gpu", WHAT);                    \
    }                                                                                          \
    extern "C" int pomdp_uninitialize_##NAME##_gpu(POMDP *pomdp) {                             \
        if (pomdp == nullptr) {                                                                \
            NOVA_ERR("pomdp_uninitialize_" #NAME "_gpu", "Invalid input.");                   \
            return NOVA_ERROR_INVALID_DATA;                                                    \
        }                                                                                      \
        return free_array<TYPE>(&pomdp->DFIELD, "pomdp_uninitialize_" #NAME "_gpu", WHAT);     \
    }

// Validation lists of pomdp_model_gpu.cu:81,128,174,220,266,313.
POMDP_ARRAY_PAIR(successors, S, d_S, int, (size_t)pomdp->n * pomdp->m * pomdp->ns,
                 pomdp->n == 0 || pomdp->m == 0 || pomdp->ns == 0, "the successor states")
POMDP_ARRAY_PAIR(state_transitions, T, d_T, float, (size_t)pomdp->n * pomdp->m * pomdp->ns,
                 pomdp->n == 0 || pomdp->m == 0 || pomdp->ns == 0, "the state transitions")
POMDP_ARRAY_PAIR(observation_transitions, O, d_O, float, (size_t)pomdp->m * pomdp->n * pomdp->z,
                 pomdp->n == 0 || pomdp->m == 0 || pomdp->z == 0, "the observation transitions")
POMDP_ARRAY_PAIR(rewards, R, d_R, float, (size_t)pomdp->n * pomdp->m,
                 pomdp->n == 0 || pomdp->m == 0, "the rewards")
POMDP_ARRAY_PAIR(nonzero_beliefs, Z, d_Z, int, (size_t)pomdp->r * pomdp->rz,
                 pomdp->r == 0 || pomdp->rz == 0, "the non-zero belief states")
POMDP_ARRAY_PAIR(belief_points, B, d_B, float, (size_t)pomdp->r * pomdp->rz,
                 pomdp->r == 0 || pomdp->rz == 0, "the belief points")

extern "C" int pomdp_initialize_gpu(POMDP *pomdp) {
    // Sum of per-array codes, as pomdp_model_gpu.cu:34-53.
    if (pomdp == nullptr) {
        NOVA_ERR("pomdp_initialize_gpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int result = 0;
    result += pomdp_initialize_successors_gpu(pomdp);
    result += pomdp_initialize_state_transitions_gpu(pomdp);
    result += pomdp_initialize_observation_transitions_gpu(pomdp);
    result += pomdp_initialize_rewards_gpu(pomdp);
    if (pomdp->r > 0) {
        result += pomdp_initialize_nonzero_beliefs_gpu(pomdp);
        result += pomdp_initialize_belief_points_gpu(pomdp);
    }
    return result;
}

extern "C" int pomdp_uninitialize_gpu(POMDP *pomdp) {
    if (pomdp == nullptr) {
        NOVA_ERR("pomdp_uninitialize_gpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int result = 0;
    result += pomdp_uninitialize_successors_gpu(pomdp);
    result += pomdp_uninitialize_state_transitions_gpu(pomdp);
    result += pomdp_uninitialize_observation_transitions_gpu(pomdp);
    result += pomdp_uninitialize_rewards_gpu(pomdp);
    if (pomdp->r > 0) {
        result += pomdp_uninitialize_nonzero_beliefs_gpu(pomdp);
        result += pomdp_uninitialize_belief_points_gpu(pomdp);
    }
    return result;
}

// ===========================================================================
// Host MDP model (mdp_model_cpu.cpp)
// ===========================================================================

extern "C" int mdp_initialize_cpu(MDP *mdp, unsigned int n, unsigned int ns, unsigned int m, float gamma,
        unsigned int horizon, float epsilon, unsigned int s0, unsigned int ng) {
    // Validation list of mdp_model_cpu.cpp:38-44.
    if (mdp == nullptr || mdp->goals != nullptr || mdp->S != nullptr ||
            mdp->T != nullptr || mdp->R != nullptr || n == 0 || ns == 0 || n < ns ||
            m == 0 || gamma < 0.0f || gamma > 1.0f || horizon == 0 || epsilon < 0.0f ||
            s0 >= n || ng >= n) {
        NOVA_ERR("mdp_initialize_cpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    mdp->n = n; mdp->ns = ns; mdp->m = m; mdp->gamma = gamma; mdp->horizon = horizon;
    mdp->epsilon = epsilon; mdp->s0 = s0; mdp->ng = ng;
    const size_t nms = (size_t)n * m * ns;
    mdp->S = new int[nms];
    mdp->T = new float[nms];
    for (size_t i = 0; i < nms; i++) { mdp->S[i] = -1; mdp->T[i] = 0.0f; }
    mdp->R = new float[(size_t)n * m]();
    mdp->goals = ng > 0 ? new unsigned int[ng]() : nullptr;
    mdp->d_goals = nullptr; mdp->d_S = nullptr; mdp->d_T = nullptr; mdp->d_R = nullptr;
    return NOVA_SUCCESS;
}

extern "C" int mdp_uninitialize_cpu(MDP *mdp) {
    if (mdp == nullptr) {
        NOVA_ERR("mdp_uninitialize_cpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    mdp->n = 0; mdp->ns = 0; mdp->m = 0; mdp->gamma = 0.0f; mdp->horizon = 0;
    mdp->epsilon = 0.0f; mdp->s0 = 0; mdp->ng = 0;
    delete[] mdp->goals; mdp->goals = nullptr;
    delete[] mdp->S; mdp->S = nullptr;
    delete[] mdp->T; mdp->T = nullptr;
    delete[] mdp->R; mdp->R = nullptr;
    return NOVA_SUCCESS;
}

// ===========================================================================
// Device MDP model (mdp_model_gpu.cu)
// ===========================================================================

#define MDP_ARRAY_PAIR(NAME, FIELD, DFIELD, TYPE, COUNT, CHECK, WHAT)                            \
    extern "C" int mdp_initialize_##NAME##_gpu(MDP *mdp) {                                     \
        if (mdp == nullptr || (CHECK) || mdp->FIELD == nullptr) {                              \
            NOVA_ERR("mdp_initialize_" #NAME "_gpu", "Invalid input.");                       \
            return NOVA_ERROR_INVALID_DATA;                                                    \
        }                                                                                      \
        return upload_array<TYPE>(&mdp->DFIELD, mdp->FIELD, (COUNT),                           \
                                  "mdp_initialize_" #NAME "_gpu", WHAT);                      \
    }                                                                                          \
    extern "C" int mdp_uninitialize_##NAME##_gpu(MDP *mdp) {                                   \
        if (mdp == nullptr) {                                                                  \
            NOVA_ERR("mdp_uninitialize_" #NAME "_gpu", "Invalid input.");                     \
            return NOVA_ERROR_INVALID_DATA;                                                    \
        }                                                                                      \
        return free_array<TYPE>(&mdp->DFIELD, "mdp_uninitialize_" #NAME "_gpu", WHAT);         \
    }

MDP_ARRAY_PAIR(successors, S, d_S, int, (size_t)mdp->n * mdp->m * mdp->ns,
               mdp->n == 0 || mdp->m == 0 || mdp->ns == 0, "the successor states")
MDP_ARRAY_PAIR(state_transitions, T, d_T, float, (size_t)mdp->n * mdp->m * mdp->ns,
               mdp->n == 0 || mdp->m == 0 || mdp->ns == 0, "the state transitions")
MDP_ARRAY_PAIR(rewards, R, d_R, float, (size_t)mdp->n * mdp->m,
               mdp->n == 0 || mdp->m == 0, "the rewards")
MDP_ARRAY_PAIR(goals, goals, d_goals, unsigned int, (size_t)mdp->ng,
               mdp->ng == 0, "the goals")

extern "C" int mdp_initialize_gpu(MDP *mdp) {
    if (mdp == nullptr) {
        NOVA_ERR("mdp_initialize_gpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int result = 0;
    result += mdp_initialize_successors_gpu(mdp);
    result += mdp_initialize_state_transitions_gpu(mdp);
    result += mdp_initialize_rewards_gpu(mdp);
    if (mdp->ng > 0) result += mdp_initialize_goals_gpu(mdp);
    return result;
}

extern "C" int mdp_uninitialize_gpu(MDP *mdp) {
    if (mdp == nullptr) {
        NOVA_ERR("mdp_uninitialize_gpu", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    int result = 0;
    result += mdp_uninitialize_successors_gpu(mdp);
    result += mdp_uninitialize_state_transitions_gpu(mdp);
    result += mdp_uninitialize_rewards_gpu(mdp);
    if (mdp->ng > 0) result += mdp_uninitialize_goals_gpu(mdp);
    return result;
}

// ===========================================================================
// Policies (pomdp_alpha_vectors.cpp, mdp_value_function.cpp)
// ===========================================================================

extern "C" int pomdp_alpha_vectors_initialize(POMDPAlphaVectors *policy, unsigned int n, unsigned int m,
        unsigned int r) {
    if (policy == nullptr || policy->Gamma != nullptr || policy->pi != nullptr || n == 0 || m == 0 || r == 0) {
        NOVA_ERR("pomdp_alpha_vectors_initialize", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    policy->n = n; policy->m = m; policy->r = r;
    policy->Gamma = new float[(size_t)r * n];
    policy->pi = new unsigned int[r];
    return NOVA_SUCCESS;
}

extern "C" int pomdp_alpha_vectors_value_and_action(const POMDPAlphaVectors *policy, const float *b,
        float &Vb, unsigned int &a) {
    // Host evaluation of a host policy, as pomdp_alpha_vectors.cpp:52-79:
    // FP32 dot products in state order, strict '<' update from -1e10.
    if (policy == nullptr || policy->n == 0 || policy->m == 0 || policy->r == 0 ||
            policy->Gamma == nullptr || policy->pi == nullptr || b == nullptr) {
        NOVA_ERR("pomdp_alpha_vectors_value_and_action", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    float best = NOVA_FLT_MIN;
    unsigned act = 0;
    for (unsigned i = 0; i < policy->r; i++) {
        float v = 0.0f;
        const float *row = policy->Gamma + (size_t)i * policy->n;
        for (unsigned s = 0; s < policy->n; s++) {
            float p = row[s] * b[s];
            v = v + p;
        }
        if (best < v) { best = v; act = policy->pi[i]; }
    }
    Vb = best;
    a = act;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_alpha_vectors_uninitialize(POMDPAlphaVectors *policy) {
    if (policy == nullptr) {
        NOVA_ERR("pomdp_alpha_vectors_uninitialize", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    policy->n = 0; policy->m = 0; policy->r = 0;
    delete[] policy->Gamma; policy->Gamma = nullptr;
    delete[] policy->pi; policy->pi = nullptr;
    return NOVA_SUCCESS;
}

extern "C" int mdp_value_function_initialize(MDPValueFunction *policy, unsigned int n, unsigned int m,
        unsigned int r) {
    if (policy == nullptr || policy->S != nullptr || policy->V != nullptr || policy->pi != nullptr ||
            n == 0 || m == 0) {
        NOVA_ERR("mdp_value_function_initialize", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    policy->n = n; policy->m = m; policy->r = r;
    if (r > 0) {
        policy->S = new unsigned int[r];
        policy->V = new float[r];
        policy->pi = new unsigned int[r];
    } else {
        policy->S = nullptr;
        policy->V = new float[n];
        policy->pi = new unsigned int[n];
    }
    return NOVA_SUCCESS;
}

extern "C" int mdp_value_function_uninitialize(MDPValueFunction *policy) {
    if (policy == nullptr) {
        NOVA_ERR("mdp_value_function_uninitialize", "Invalid input.");
        return NOVA_ERROR_INVALID_DATA;
    }
    policy->n = 0; policy->m = 0; policy->r = 0;
    delete[] policy->S; policy->S = nullptr;
    delete[] policy->V; policy->V = nullptr;
    delete[] policy->pi; policy->pi = nullptr;
    return NOVA_SUCCESS;
}

// ===========================================================================
// Library status and test hooks
// ===========================================================================

extern "C" void nova_gb300_inject_fault(unsigned int kind, unsigned int count) {
    g_fault_kind.store(count == 0 ? 0u : kind);
    g_fault_countdown.store(count);
}

extern "C" unsigned long long nova_gb300_kernel_launches(void) { return launch_count(); }

extern "C" int nova_gb300_device_status(unsigned int *deviceError) {
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) {
        cudaGetLastError();
        if (deviceError) *deviceError = 0;
        return 0;
    }
    if (deviceError) *deviceError = read_and_clear_device_error();
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) return 0;
    return (prop.major == 10 && prop.minor == 3) ? 1 : 0;
}
