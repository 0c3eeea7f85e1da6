// nova-gb300: many independent PBVI solves at once.
//
// Small POMDPs leave most of a GB300 idle when solved one after another:
// their kernels are a few thousand threads each and every update ends in a
// host synchronisation. Here a pool of host threads takes POMDPs from a
// shared queue (largest estimated scoring work first) and solves each with
// the ordinary solver (same kernels, same results as pomdp_pbvi_execute_gpu).
// The library is built with per-thread default streams, so the solves of
// different host threads run concurrently on the device.

#include "common.h"
#include "pbvi.h"

#include <algorithm>
#include <atomic>
#include <mutex>
#include <shared_mutex>
#include <thread>
#include <vector>

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_gpu.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>
#include <nova/nova_gb300.h>

using nova::POMDP;
using nova::POMDPPBVIGPU;
using nova::POMDPAlphaVectors;

namespace {

// Calls other than the updates (which lock for themselves) hold the capture
// lock shared, so that no allocation or device synchronisation of this
// thread overlaps another solver's graph capture.
int solve_one(const POMDP *pomdp, POMDPPBVIGPU *pbvi, POMDPAlphaVectors *policy, unsigned scoring, bool graph) {
    using Shared = std::shared_lock<std::shared_mutex>;
    int rc;
    {
        Shared lock(nova_gb300::capture_lock());
        rc = pomdp_pbvi_initialize_gpu(pomdp, pbvi);
        if (rc != NOVA_SUCCESS) return rc;
        if ((rc = pomdp_pbvi_set_scoring_gpu(pbvi, scoring)) != NOVA_SUCCESS ||
                (rc = pomdp_pbvi_set_graph_gpu(pbvi, graph ? 1u : 0u)) != NOVA_SUCCESS) {
            pomdp_pbvi_uninitialize_gpu(pomdp, pbvi);
            return rc;
        }
    }
    while (pbvi->currentHorizon < pomdp->horizon) {
        rc = pomdp_pbvi_update_gpu(pomdp, pbvi);
        if (rc != NOVA_SUCCESS) {
            Shared lock(nova_gb300::capture_lock());
            pomdp_pbvi_uninitialize_gpu(pomdp, pbvi);
            return rc;
        }
    }
    Shared lock(nova_gb300::capture_lock());
    rc = pomdp_pbvi_get_policy_gpu(pomdp, pbvi, policy);
    const int rc2 = pomdp_pbvi_uninitialize_gpu(pomdp, pbvi);
    return rc != NOVA_SUCCESS ? rc : rc2;
}

}  // namespace

static int execute_batched(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                           POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
                           unsigned int hostThreads, bool graph, const char *fn) {
    if (pomdps == nullptr || solvers == nullptr || policies == nullptr || count == 0 ||
            (scoring != NOVA_SCORING_EXACT && scoring != NOVA_SCORING_BF16 && scoring != NOVA_SCORING_FP16)) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    for (unsigned k = 0; k < count; k++) {
        if (pomdps[k] == nullptr || solvers[k] == nullptr || policies[k] == nullptr) {
            NOVA_ERR(fn, "Invalid arguments.");
            return NOVA_ERROR_INVALID_DATA;
        }
        for (unsigned q = 0; q < k; q++)
            if (solvers[q] == solvers[k]) {
                NOVA_ERR(fn, "Invalid arguments: a solver struct appears twice.");
                return NOVA_ERROR_INVALID_DATA;
            }
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "No usable current CUDA device.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    // Largest scoring work (r^2 n m z) first, so the long solves start early.
    std::vector<unsigned> order(count);
    for (unsigned k = 0; k < count; k++) order[k] = k;
    auto work = [&](unsigned k) {
        const POMDP *p = pomdps[k];
        return (double)p->r * p->r * p->n * p->m * p->z * p->horizon;
    };
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) { return work(a) > work(b); });
    unsigned threads = hostThreads ? hostThreads : std::min(count, 16u);
    threads = std::max(1u, std::min(threads, count));
    std::atomic<unsigned> next{0};
    std::atomic<int> firstError{NOVA_SUCCESS};
    auto worker = [&]() {
        if (cudaSetDevice(dev) != cudaSuccess) {
            cudaGetLastError();
            int expected = NOVA_SUCCESS;
            firstError.compare_exchange_strong(expected, NOVA_ERROR_INVALID_CUDA_PARAM);
            return;
        }
        for (unsigned k = next.fetch_add(1); k < count; k = next.fetch_add(1)) {
            const unsigned p = order[k];
            const int rc = solve_one(pomdps[p], solvers[p], policies[p], scoring, graph);
            if (rc != NOVA_SUCCESS) {
                int expected = NOVA_SUCCESS;
                firstError.compare_exchange_strong(expected, rc);
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; t++) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    return firstError.load();
}

extern "C" int pomdp_pbvi_execute_batched_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                                              POMDPAlphaVectors *const *policies, unsigned int count,
                                              unsigned int scoring, unsigned int hostThreads) {
    return execute_batched(pomdps, solvers, policies, count, scoring, hostThreads, false,
                           "pomdp_pbvi_execute_batched_gpu");
}

extern "C" int pomdp_pbvi_execute_batched_graph_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                                                    POMDPAlphaVectors *const *policies, unsigned int count,
                                                    unsigned int scoring, unsigned int hostThreads) {
    return execute_batched(pomdps, solvers, policies, count, scoring, hostThreads, true,
                           "pomdp_pbvi_execute_batched_graph_gpu");
}
