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

static int validate_batch(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                          POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
                          const char *fn) {
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
    return NOVA_SUCCESS;
}

static int execute_batched(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                           POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
                           unsigned int hostThreads, bool graph, const char *fn) {
    const int rcValid = validate_batch(pomdps, solvers, policies, count, scoring, fn);
    if (rcValid != NOVA_SUCCESS) return rcValid;
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

// ---------------------------------------------------------------------------
// Lock-step batched solve: one persistent scoring launch per backup for all
// solvers of the batch.
//
//   1. Warm-up (pool of host threads, the ordinary update): each solver runs
//      updates until its tensor-core schedule is fixed (its first
//      tensor-core updates tune it). A tuned solver whose exact scan could
//      plausibly be cheaper then times one update with exact scoring and
//      keeps exact scoring if that is cheaper per unique alpha than its best
//      tensor-core schedule.
//   2. Lock-step backups (one host thread, one stream per solver): every
//      backup of every solver runs without host read-backs (the fixed update
//      of graph mode); each solver's projection table and alpha packing are
//      queued on its own stream, one persistent tcgen05 launch per list
//      length scores the work units of all tensor-core solvers from a device
//      table of their tensor maps and shapes, and each solver's merge, exact
//      scan and assembly follow on its stream. The table is rebuilt only when
//      the set of solvers still running changes.
//   3. Policies are read back and the solvers released.
// The batch runs in waves whose solvers' tables fit in device memory
// together, largest first. Results are bit-identical to solving each POMDP
// alone.
// ---------------------------------------------------------------------------

namespace {

using nova_gb300::BackupEngine;

struct LockstepSolver {
    const POMDP *pomdp = nullptr;
    POMDPPBVIGPU *pbvi = nullptr;
    BackupEngine *eng = nullptr;
    cudaStream_t stream = nullptr, savedStream = nullptr;
    cudaEvent_t prep = nullptr;
    bool tensor = false;     // scores on the tensor cores (else exactly)
    bool lockstep = false;   // runs its remaining updates in lock-step
    int rc = NOVA_SUCCESS;
};

// Phase 1 for one solver: initialize, warm up, choose the scoring form.
void warm_up(LockstepSolver &S, unsigned scoring) {
    using Shared = std::shared_lock<std::shared_mutex>;
    int rc;
    {
        Shared lock(nova_gb300::capture_lock());
        rc = pomdp_pbvi_initialize_gpu(S.pomdp, S.pbvi);
        if (rc == NOVA_SUCCESS) rc = pomdp_pbvi_set_scoring_gpu(S.pbvi, scoring);
    }
    if (rc != NOVA_SUCCESS) { S.rc = rc; return; }
    const unsigned H = S.pomdp->horizon;
    auto ready = [&](const BackupEngine *e) {
        if (e == nullptr) return false;
        if (scoring == NOVA_SCORING_EXACT || e->tcUnavailable || !nova_gb300::tc_supported(e->md)) return true;
        return nova_gb300::tc_schedule_fixed(*e);
    };
    while (S.pbvi->currentHorizon < H && !ready(nova_gb300::pbvi_gpu_engine(S.pbvi))) {
        if ((rc = pomdp_pbvi_update_gpu(S.pomdp, S.pbvi)) != NOVA_SUCCESS) { S.rc = rc; return; }
    }
    BackupEngine *e = nova_gb300::pbvi_gpu_engine(S.pbvi);
    if (e == nullptr || S.pbvi->currentHorizon >= H) return;
    S.eng = e;
    S.tensor = scoring != NOVA_SCORING_EXACT && e->tc != nullptr && !e->tcUnavailable &&
               nova_gb300::tc_schedule_fixed(*e) && e->md.r >= BackupEngine::kTcMinUnique;
    const float tcCost = S.tensor ? nova_gb300::tc_tuned_cost(*e) : -1.0f;
    // The exact scan reads rz table entries per (row, alpha); at about 2.2e12
    // such reads per second (the n=4096 workload) it is worth a timed trial
    // only when that estimate is within twice the tuned tensor-core time.
    const double nU = (double)std::max(1u, e->stats.uniqueAlphas);
    const double exactEstimateMs = (double)e->md.m * e->md.z * e->md.r * nU * e->md.rz / 2.2e12 * 1e3;
    if (tcCost > 0.0f && exactEstimateMs < 2.0 * (double)tcCost * nU && S.pbvi->currentHorizon < H) {
        if ((rc = pomdp_pbvi_set_scoring_gpu(S.pbvi, NOVA_SCORING_EXACT)) == NOVA_SUCCESS)
            rc = pomdp_pbvi_update_gpu(S.pomdp, S.pbvi);
        if (rc == NOVA_SUCCESS) {
            const auto &st = e->stats;
            const float exactCost = (st.msScore + st.msRescore) / (float)std::max(1u, st.uniqueAlphas);
            if (exactCost < tcCost) S.tensor = false;
            rc = pomdp_pbvi_set_scoring_gpu(S.pbvi, scoring);
        }
        if (rc != NOVA_SUCCESS) { S.rc = rc; return; }
    }
    S.lockstep = S.pbvi->currentHorizon < H;
}

// Phase 3 for one solver: any remaining ordinary updates, the policy, release.
int finish_solver(LockstepSolver &S, POMDPAlphaVectors *policy) {
    using Shared = std::shared_lock<std::shared_mutex>;
    int rc = S.rc;
    while (rc == NOVA_SUCCESS && S.pbvi->currentHorizon < S.pomdp->horizon)
        rc = pomdp_pbvi_update_gpu(S.pomdp, S.pbvi);
    Shared lock(nova_gb300::capture_lock());
    if (rc == NOVA_SUCCESS) rc = pomdp_pbvi_get_policy_gpu(S.pomdp, S.pbvi, policy);
    const int rc2 = pomdp_pbvi_uninitialize_gpu(S.pomdp, S.pbvi);
    return rc != NOVA_SUCCESS ? rc : rc2;
}

// Device memory one solver of the batch holds while it runs (scoring
// operand, projection table, candidate lists, coefficient tables, alpha sets).
double solver_footprint(const POMDP *p) {
    const double mz = (double)p->m * p->z, r = p->r, n = p->n;
    const double rPad = (double)((p->r + 127) / 128 * 128), nPad = (double)((p->n + 63) / 64 * 64);
    const double operand = mz * rPad * nPad * 2.0;
    const double table = mz * nPad * (double)((p->r + 31) / 32 * 32) * 4.0;
    const double lists = mz * r * 8.0 * (32.0 * 8.0 + 4.0) + mz * r * 16.0;
    const double coef = 2.0 * n * p->m * p->ns * p->z * 4.0;
    const double alphas = 5.0 * r * n * 4.0 + mz * r * 16.0;
    return operand + table + lists + coef + alphas;
}

int execute_lockstep_wave(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                          POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
                          unsigned int hostThreads, int dev, const char *fn) {
    std::vector<LockstepSolver> S(count);
    for (unsigned k = 0; k < count; k++) { S[k].pomdp = pomdps[k]; S[k].pbvi = solvers[k]; }
    // ---- 1. warm-up on a pool of host threads ----
    {
        const unsigned threads = std::max(1u, std::min(hostThreads ? hostThreads : std::min(count, 16u), count));
        std::atomic<unsigned> next{0};
        auto worker = [&]() {
            if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return; }
            for (unsigned k = next.fetch_add(1); k < count; k = next.fetch_add(1)) warm_up(S[k], scoring);
        };
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < threads; t++) pool.emplace_back(worker);
        worker();
        for (auto &t : pool) t.join();
    }
    int rc = nova_gb300::sync_device(fn);
    // ---- 2. lock-step backups ----
    std::vector<unsigned> lock;
    for (unsigned k = 0; k < count && rc == NOVA_SUCCESS; k++) {
        LockstepSolver &L = S[k];
        if (L.rc != NOVA_SUCCESS || !L.lockstep) continue;
        if (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&L.prep, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            L.lockstep = false;
            continue;
        }
        L.savedStream = L.eng->stream;
        L.eng->stream = L.stream;
        if (L.eng->fixed_setup(fn) != NOVA_SUCCESS || !L.eng->ensure_proj(L.eng->md.r) ||
                (L.tensor && !L.eng->fixed_ready())) {
            cudaStreamSynchronize(L.stream);
            L.eng->stream = L.savedStream;
            L.lockstep = false;   // ordinary updates in phase 3
            continue;
        }
        lock.push_back(k);
    }
    cudaStream_t gemmStream = nullptr;
    cudaEvent_t scored = nullptr;
    if (rc == NOVA_SUCCESS && !lock.empty() &&
            (cudaStreamCreateWithFlags(&gemmStream, cudaStreamNonBlocking) != cudaSuccess ||
             cudaEventCreateWithFlags(&scored, cudaEventDisableTiming) != cudaSuccess)) {
        cudaGetLastError();
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
    nova_gb300::TcBatch *batch = nullptr;
    std::vector<BackupEngine *> batchEngines;
    while (rc == NOVA_SUCCESS) {
        std::vector<unsigned> active;
        for (unsigned k : lock)
            if (S[k].pbvi->currentHorizon < S[k].pomdp->horizon) active.push_back(k);
        if (active.empty()) break;
        std::vector<BackupEngine *> tensorEngines;
        for (unsigned k : active) {
            LockstepSolver &L = S[k];
            const bool even = (L.pbvi->currentHorizon % 2u) == 0u;
            const float *src = even ? L.pbvi->d_Gamma : L.pbvi->d_GammaPrime;
            if ((rc = L.eng->fixed_pre(src, L.tensor, fn)) != NOVA_SUCCESS) break;
            if (L.tensor) {
                cudaEventRecord(L.prep, L.stream);
                cudaStreamWaitEvent(gemmStream, L.prep, 0);
                tensorEngines.push_back(L.eng);
            }
        }
        if (rc != NOVA_SUCCESS) break;
        if (!tensorEngines.empty()) {
            if (batch == nullptr || tensorEngines != batchEngines) {
                // The table is built from the prepared launches (host data);
                // the previous table may still be read by a launch in flight.
                if (batch != nullptr) {
                    cudaStreamSynchronize(gemmStream);
                    nova_gb300::tc_batch_release(batch);
                    batch = nullptr;
                }
                if ((rc = nova_gb300::tc_batch_create(tensorEngines.data(), (unsigned)tensorEngines.size(), &batch,
                                                      fn)) != NOVA_SUCCESS)
                    break;
                batchEngines = tensorEngines;
            }
            if ((rc = nova_gb300::tc_batch_gemm(batch, gemmStream, fn)) != NOVA_SUCCESS) break;
            cudaEventRecord(scored, gemmStream);
        }
        for (unsigned k : active) {
            LockstepSolver &L = S[k];
            const bool even = (L.pbvi->currentHorizon % 2u) == 0u;
            const float *src = even ? L.pbvi->d_Gamma : L.pbvi->d_GammaPrime;
            float *dst = even ? L.pbvi->d_GammaPrime : L.pbvi->d_Gamma;
            if (L.tensor) cudaStreamWaitEvent(L.stream, scored, 0);
            if ((rc = L.eng->fixed_post(src, dst, L.pbvi->d_pi, L.tensor, fn)) != NOVA_SUCCESS) break;
            L.pbvi->currentHorizon++;
        }
    }
    const int rcSync = nova_gb300::sync_device(fn);
    if (rc == NOVA_SUCCESS) rc = rcSync;
    if (rc == NOVA_SUCCESS && nova_gb300::tc_device_error() != 0) {
        NOVA_ERR(fn, "A device-side wait timed out; results are invalid.");
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (batch != nullptr) nova_gb300::tc_batch_release(batch);
    for (unsigned k : lock) {
        S[k].eng->stream = S[k].savedStream;
        S[k].eng->stats.horizon = S[k].pbvi->currentHorizon;
    }
    for (auto &L : S) {
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.prep) cudaEventDestroy(L.prep);
    }
    if (gemmStream) cudaStreamDestroy(gemmStream);
    if (scored) cudaEventDestroy(scored);
    // ---- 3. remaining ordinary updates, policies, release ----
    int first = rc;
    for (unsigned k = 0; k < count; k++) {
        if (rc != NOVA_SUCCESS && S[k].rc == NOVA_SUCCESS) S[k].rc = rc;
        const int r = finish_solver(S[k], policies[k]);
        if (first == NOVA_SUCCESS && r != NOVA_SUCCESS) first = r;
    }
    return first;
}

// The batch in waves that fit in device memory together (every solver of a
// wave holds its tables at once), largest solvers first.
int execute_lockstep(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers, POMDPAlphaVectors *const *policies,
                     unsigned int count, unsigned int scoring, unsigned int hostThreads, const char *fn) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "No usable current CUDA device.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    std::vector<unsigned> order(count);
    for (unsigned k = 0; k < count; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](unsigned a, unsigned b) {
        return solver_footprint(pomdps[a]) > solver_footprint(pomdps[b]);
    });
    size_t freeB = 0, totalB = 0;
    cudaMemGetInfo(&freeB, &totalB);
    const double budget = 0.6 * (double)freeB;
    int first = NOVA_SUCCESS;
    for (unsigned k0 = 0; k0 < count;) {
        double used = 0.0;
        unsigned k1 = k0;
        while (k1 < count && (k1 == k0 || used + solver_footprint(pomdps[order[k1]]) <= budget))
            used += solver_footprint(pomdps[order[k1++]]);
        std::vector<const POMDP *> P;
        std::vector<POMDPPBVIGPU *> G;
        std::vector<POMDPAlphaVectors *> A;
        for (unsigned k = k0; k < k1; k++) {
            P.push_back(pomdps[order[k]]);
            G.push_back(solvers[order[k]]);
            A.push_back(policies[order[k]]);
        }
        const int rc = execute_lockstep_wave(P.data(), G.data(), A.data(), k1 - k0, scoring, hostThreads, dev, fn);
        if (first == NOVA_SUCCESS) first = rc;
        k0 = k1;
    }
    return first;
}

}  // namespace

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

extern "C" int pomdp_pbvi_execute_batched_persistent_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
                                                         POMDPAlphaVectors *const *policies, unsigned int count,
                                                         unsigned int scoring, unsigned int hostThreads) {
    static const char *fn = "pomdp_pbvi_execute_batched_persistent_gpu";
    const int rc = validate_batch(pomdps, solvers, policies, count, scoring, fn);
    if (rc != NOVA_SUCCESS) return rc;
    return execute_lockstep(pomdps, solvers, policies, count, scoring, hostThreads, fn);
}
