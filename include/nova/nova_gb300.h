/*
 * nova-gb300: additive entry points (no counterpart in the reference).
 *
 * The reference's own entry points keep their exact semantics; everything
 * here is new and optional. All functions are synchronous and return NOVA_*
 * status codes.
 */
#ifndef NOVA_GB300_H
#define NOVA_GB300_H

#include <nova/nova_abi.h>
#include <nova/mdp/mdp.h>
#include <nova/mdp/algorithms/mdp_vi_gpu.h>
#include <nova/mdp/policies/mdp_value_function.h>
#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_gpu.h>
#include <nova/pomdp/policies/pomdp_alpha_vectors.h>

NOVA_NS_BEGIN

/* Belief-scoring modes of the PBVI / Perseus backup.
 *  NOVA_SCORING_EXACT: every candidate alpha is scored in FP32 in the
 *      reference's operation order (bit-identical to pomdp_pbvi_cpu.cpp:37-103).
 *  NOVA_SCORING_BF16: tcgen05 tensor cores score all alphas with BF16
 *      operands and FP32 accumulation: the belief operand in one BF16 term,
 *      the alphas as a pair of BF16 terms (hi + lo, 16 significant bits), so
 *      the scoring GEMM does twice FP16's work; every alpha within a proven
 *      error bound of the best is re-scored in the exact FP32 order, so the
 *      argmax equals EXACT's.
 *  NOVA_SCORING_FP16: one FP16 term per operand (per-belief power-of-two
 *      scaling keeps them in range), half BF16's GEMM work; the default. */
#define NOVA_SCORING_EXACT 0u
#define NOVA_SCORING_BF16  1u
#define NOVA_SCORING_FP16  2u

/* Select the scoring mode used by later pomdp_pbvi_update_gpu calls on this
 * solver struct. The default is NOVA_SCORING_FP16 (the fastest). Tensor-core
 * scoring engages once 32 distinct alphas exist and the
 * projection table fits in device memory; otherwise rows are scored exactly.
 * All modes give bit-identical results. */
NOVA_API int pomdp_pbvi_set_scoring_gpu(POMDPPBVIGPU *pbvi, unsigned int mode);

/* Projection table of a GPU PBVI solver (new in nova-gb300; replaces no
 * reference entry point). The table holds fl(gamma * sum_l C1 * alpha(S))
 * for every (action, observation, state, unique alpha): 4*m*z*n*|Gamma|
 * bytes (68.7 GB at n = 4096, m = 16, z = 32, |Gamma| = 8192). Exact scores
 * of the tensor-core candidates, the exact scan and the assembly read it.
 *  NOVA_PBVI_TABLE_AUTO (default): built when it fits in free device memory
 *        (with 1 GB to spare).
 *  NOVA_PBVI_TABLE_NEVER: never built (an existing one is freed). Tensor-core
 *        updates then re-score their candidates, score the rows their margin
 *        leaves open and assemble the new alphas straight from the model and
 *        the alphas; the exact form scores every (belief, action) pair from
 *        the alphas. Results are bit-identical either way; this is also what
 *        AUTO does when the table does not fit.
 * Returns NOVA_ERROR_INVALID_DATA for a null or uninitialized solver or an
 * unknown mode. */
#define NOVA_PBVI_TABLE_AUTO  0u
#define NOVA_PBVI_TABLE_NEVER 1u
NOVA_API int pomdp_pbvi_set_table_gpu(POMDPPBVIGPU *pbvi, unsigned int mode);

/* Graph mode for later pomdp_pbvi_update_gpu calls on this solver (default
 * off). Once the solver scores on the tensor cores with a fixed schedule (its
 * first tensor-core updates tune it), each update replays a CUDA graph of the
 * whole backup: every alpha is scored as its own (no duplicate removal, the
 * same argmax by the lowest index), the exact scan is sized on the device,
 * and nothing is read back to the host inside the update; one graph per
 * direction (Gamma -> GammaPrime and back) is captured on first use. Updates
 * stay synchronous and give the same results; their statistics keep only the
 * horizon, scoring mode, alpha count and kernel count. */
NOVA_API int pomdp_pbvi_set_graph_gpu(POMDPPBVIGPU *pbvi, unsigned int enable);

/* Per-update counters of the last pomdp_pbvi_update_gpu on this solver. */
typedef struct NovaPBVIStats {
    unsigned int horizon;          /* currentHorizon after the update */
    unsigned int scoring;          /* mode actually used */
    unsigned int uniqueAlphas;     /* distinct rows of the input Gamma */
    unsigned int rowsMultiCand;    /* (belief, action, obs) rows re-scored exactly */
    unsigned int rowsOverflow;     /* (belief, action) pairs scored exactly in full */
    unsigned int candidates;       /* total alphas re-scored in FP32 */
    float msDedup, msProject, msScore, msRescore, msActions, msAssemble, msTotal;
    float msGemm;                  /* the tensor-core scoring kernel alone (0 if not run) */
    unsigned int launches;         /* kernels this library launched for the update */
    unsigned int tcGroups;         /* alpha groups of the tensor-core launch (0 if not run) */
} NovaPBVIStats;

NOVA_API int pomdp_pbvi_get_stats_gpu(const POMDPPBVIGPU *pbvi, NovaPBVIStats *stats);

/* Per-belief detail of the last pomdp_pbvi_update_gpu on this solver, when
 * it scored on the tensor cores (NovaPBVIStats.tcGroups != 0): for belief i,
 * candidates[i] = alphas re-scored exactly in the FP32 order because their
 * tensor-core score lay within the proven margin of the best, summed over
 * the belief's (action, observation) rows, and exactRows[i] = its rows that
 * were scanned exactly over every alpha. Host arrays of r entries. A test
 * and measurement aid for the scoring path of pomdp_pbvi_cpu.cpp:37-103; no
 * reference counterpart. NOVA_ERROR_INVALID_DATA if the last update did not
 * use the tensor cores (or ran as a graph replay). */
NOVA_API int pomdp_pbvi_row_detail_gpu(const POMDPPBVIGPU *pbvi, unsigned int *candidates,
        unsigned int *exactRows);

/* V(b) = max_i Gamma_i . b over the solver's current device Gamma (the one
 * get_policy would return), reduced in FP64 on the device. b is a dense host
 * array of n floats; *a receives pi of the maximising alpha (lowest index on
 * ties). Replaces, for device-resident policies, the host evaluation in
 * pomdp_alpha_vectors.cpp:52-79. */
NOVA_API int pomdp_pbvi_value_gpu(const POMDP *pomdp, const POMDPPBVIGPU *pbvi,
        const float *b, double *Vb, unsigned int *a);

/* One pomdp_pbvi_update_gpu that also records its selections into caller
 * device arrays: d_action[i] = the action whose alpha became GammaPrime[i]
 * (pi[i]) and d_select[i*z + o] = the alpha index j* taken for (i, that
 * action, o), i.e. the argmax results of pomdp_pbvi_cpu.cpp:37-103 (lowest
 * index among equal rows). No reference counterpart. */
NOVA_API int pomdp_pbvi_update_record_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi,
        unsigned int *d_action, unsigned int *d_select);

/* horizon recorded updates from the solver's current state. Before update t
 * with t % checkpointEvery == 0 the current Gamma is copied to
 * d_checkpoints[t / checkpointEvery] ([ceil(horizon/checkpointEvery)][r][n]);
 * the selections of update t go to d_actions[t] ([horizon][r]) and
 * d_selects[t] ([horizon][r][z]). No reference counterpart. */
NOVA_API int pomdp_pbvi_execute_recorded_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi,
        unsigned int horizon, unsigned int checkpointEvery, float *d_checkpoints,
        unsigned int *d_actions, unsigned int *d_selects);

/* Reverse mode of horizon recorded backups (selections held fixed):
 * V(b) = max_i b . Gamma_H[i] (FP64, lowest index on ties) and its gradient
 * with respect to the model's R (d_dR [n][m]), T (d_dT [n][m][ns]) and O
 * (d_dO [m][n][z]), all FP64 device arrays, plus optionally Gamma_0
 * (d_dGamma0 [r][n]). Alphas between checkpoints are recomputed in FP32 in
 * the reference's operation order, bit-identical to the forward pass. The
 * model's device arrays must be those the recorded forward ran on. No
 * reference counterpart (the reference has no differentiation). */
NOVA_API int pomdp_pbvi_adjoint_gpu(const POMDP *pomdp, unsigned int horizon,
        unsigned int checkpointEvery, const float *d_checkpoints, const unsigned int *d_actions,
        const unsigned int *d_selects, const float *d_b, double *d_dR, double *d_dT, double *d_dO,
        double *d_dGamma0, double *Vb, unsigned int *bestAlpha);

/* V(b) of the alpha set that horizon recorded backups make from d_Gamma0
 * ([r][n], FP32, device), recomputed in FP64 with the recorded selections
 * held fixed (d_actions [horizon][r], d_selects [horizon][r][z] as
 * pomdp_pbvi_execute_recorded_gpu writes them): every backup
 * Gamma_t[i](s) = R(s,a) + gamma sum_l T(s,a,l) sum_o O(a,S,o) Gamma_{t-1}[j_o](S)
 * (pomdp_pbvi_cpu.cpp:37-162 with its argmax results fixed) runs in FP64
 * from the model's device arrays. *Vb = d_b . Gamma_H[alpha] for alpha < r
 * (the FP32 run's own maximising alpha, so that only the arithmetic
 * differs), else the FP64 maximum from -1e10 with the lowest index on ties
 * (pomdp_alpha_vectors.cpp:52-79); *bestAlpha (may be NULL) receives the
 * row used. The FP64 reference of a solve's V(b0); no reference
 * counterpart. */
NOVA_API int pomdp_pbvi_value_replay_f64_gpu(const POMDP *pomdp, unsigned int horizon, const float *d_Gamma0,
        const unsigned int *d_actions, const unsigned int *d_selects, const float *d_b, unsigned int alpha,
        double *Vb, unsigned int *bestAlpha);

/* Solve count independent POMDPs, each as pomdp_pbvi_execute_gpu would
 * (initialize, `horizon` updates with the given NOVA_SCORING_* mode,
 * get_policy into policies[k], uninitialize), with identical results. A pool
 * of hostThreads host threads (0: min(count, 16)) takes the POMDPs largest
 * first; every thread drives its own per-thread default stream, so small
 * solves overlap on the device. Every POMDP must already have its device
 * copy (pomdp_initialize_gpu) and every solver struct must be distinct.
 * Returns the first failing solve's code (the others still run). No
 * reference counterpart. */
NOVA_API int pomdp_pbvi_execute_batched_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
        POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
        unsigned int hostThreads);

/* As pomdp_pbvi_execute_batched_gpu with every solver in graph mode
 * (pomdp_pbvi_set_graph_gpu): after its first tensor-core updates, each
 * solve's horizon loop replays two captured CUDA graphs. Same results. No
 * reference counterpart. */
NOVA_API int pomdp_pbvi_execute_batched_graph_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
        POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
        unsigned int hostThreads);

/* As pomdp_pbvi_execute_batched_gpu (same arguments, same results), with the
 * solvers' backups run in lock-step after a warm-up: each solver first runs
 * ordinary updates on a pool of hostThreads host threads until its
 * tensor-core schedule is tuned (a tuned solver whose exact scan could be
 * cheaper also times one update with exact scoring and keeps it if it is);
 * from then on every backup of every solver is queued without host
 * read-backs on a stream of its own, and one persistent tcgen05 scoring
 * launch (per candidate-list length) draws the work units of all
 * tensor-core solvers from a device table of their tensor maps, shapes and
 * candidate arrays. The batch runs in waves whose solvers fit in device
 * memory together. Replaces the reference's one-solve-per-call structure
 * (pomdp_pbvi_gpu.cu:361-441) for batches; no reference counterpart. */
NOVA_API int pomdp_pbvi_execute_batched_persistent_gpu(const POMDP *const *pomdps, POMDPPBVIGPU *const *solvers,
        POMDPAlphaVectors *const *policies, unsigned int count, unsigned int scoring,
        unsigned int hostThreads);

/* Random belief expansion seeds libc rand() with time(nullptr), as the
 * reference does (pomdp_expand_cpu.cpp:91, pomdp_expand_gpu.cu:139). With
 * fixed != 0, later expansions call srand(seed) instead, so runs repeat;
 * fixed == 0 restores the clock. No reference counterpart. */
NOVA_API int nova_gb300_expand_seed(unsigned int fixed, unsigned int seed);

/* V(b) and the action for count dense beliefs at once (d_B [count][n]) over a
 * device-resident policy (d_Gamma [r][n], d_pi [r]): each result has the bits
 * of pomdp_alpha_vectors_value_and_action (pomdp_alpha_vectors.cpp:52-79):
 * FP32 sums in state order, maximum from -1e10 with the lowest index on
 * ties, action pi of that alpha. d_V [count], d_a [count]. Replaces the
 * reference's one-belief-at-a-time host evaluation; no reference
 * counterpart for the batch. */
NOVA_API int pomdp_alpha_vectors_value_batched_gpu(const float *d_Gamma, const unsigned int *d_pi,
        unsigned int r, unsigned int n, const float *d_B, unsigned int count, float *d_V,
        unsigned int *d_a);

/* The same with the policy and beliefs in host memory (policy as returned by
 * get_policy, B [count][n] host); V [count], a [count] host. */
NOVA_API int pomdp_alpha_vectors_value_and_action_batched(const POMDPAlphaVectors *policy,
        const float *B, unsigned int count, float *V, unsigned int *a);

/* Load nova's raw comma-separated POMDP / MDP files (the layout read by
 * FileLoader.load_raw_pomdp / load_raw_mdp, python/nova/file_loader.py:74-209)
 * into a struct whose arrays are still null; the arrays are allocated as
 * pomdp_initialize_cpu / mdp_initialize_cpu do. Of the file's k reward
 * functions, rewardIndex is kept (the reference's default keeps the first). */
NOVA_API int nova_load_raw_pomdp(const char *path, POMDP *pomdp, unsigned int rewardIndex);
NOVA_API int nova_load_raw_mdp(const char *path, MDP *mdp, unsigned int rewardIndex);

/* Cassandra-format POMDP file into an uninitialized POMDP (host arrays, as
 * pomdp_initialize_cpu allocates them), with the rules of the reference's
 * FileLoader.load_cassandra (python/nova/file_loader.py:211-588): one belief
 * (r = 1) from start / start include / start exclude, successor lists in
 * statement order, R(s,a) the mean of each reward statement's numbers, the
 * horizon from the reward range. Rmin and Rmax (may be NULL) receive the
 * extreme rewards in double precision, as the reference's loader keeps them.
 * NOVA_ERROR_INVALID_DATA where the reference fails to load the file. */
NOVA_API int nova_load_cassandra_pomdp(const char *path, POMDP *pomdp, double *Rmin, double *Rmax);

/* Value iteration until the Bellman residual max_s |V'(s) - V(s)|, computed
 * in FP64 on the device after every sweep, drops below tol, or maxSweeps
 * sweeps ran. The reference's VI has no convergence test (mdp_vi_gpu.cu:163-221
 * runs exactly `horizon` sweeps). The policy is filled as by
 * mdp_vi_get_policy_gpu. */
NOVA_API int mdp_vi_execute_until_converged_gpu(const MDP *mdp, MDPVIGPU *vi,
        MDPValueFunction *policy, double tol, unsigned int maxSweeps,
        unsigned int *sweeps, double *residual);

/* Residual max_s |V'(s) - V(s)| in FP64 of the last sweep made by
 * mdp_vi_update_gpu on this solver. */
NOVA_API int mdp_vi_residual_gpu(const MDP *mdp, const MDPVIGPU *vi, double *residual);

/* Sweep kernel selection. Replaces nothing in the reference (its sweep,
 * mdp_vi_gpu.cu:37-87, has one form). When every (s, a) row lists its valid
 * successors in ascending state order, the sweep can stage V in shared-memory
 * tiles and add each row's products tile by tile, which is the reference's
 * own order (mdp_vi_cpu.cpp:45-52), so results stay bit-identical; other
 * models use the per-row gather sweep. A solver builds its tile plan (8 bytes
 * per successor entry) at its first sweep after initialize, from the model's
 * S, T and gamma as they are then.
 *  mode: NOVA_VI_TILING_AUTO (default: tiled for models with at least 2^22
 *        successor entries), NOVA_VI_TILING_ALWAYS (whenever the model
 *        qualifies), NOVA_VI_TILING_NEVER.
 *  tileStates: states per shared-memory tile of V, a multiple of 4 in
 *        [64, 16384], or 0 for the default: the largest tile of 8192 to
 *        10240 states (steps of 256) that needs no more rounds of source
 *        blocks over the SMs than 8192 states does.
 * The setting is process-wide and applies to plans built after the call. */
#define NOVA_VI_TILING_AUTO   0u
#define NOVA_VI_TILING_ALWAYS 1u
#define NOVA_VI_TILING_NEVER  2u
NOVA_API int mdp_vi_set_tiling_gpu(unsigned int mode, unsigned int tileStates);

/* Sweep kernel of an initialized solver struct (an MDPVIGPU or MDPVICPU):
 * 0 = no sweep yet, 1 = tiled, 2 = per-row gather. With vi == NULL, the
 * status of the plan built last in this process. */
NOVA_API int mdp_vi_tiling_status_gpu(const void *vi, unsigned int *status);

/* Library self-description: 1 if the library was built for sm_103a and a
 * device is present, 0 otherwise; *deviceError receives (and clears) the
 * device-side error word that bounded waits set instead of hanging. */
NOVA_API int nova_gb300_device_status(unsigned int *deviceError);

/* Allocation-free V(b) for an alpha-vector policy already in device memory.
 * This entry point has no counterpart in the reference. It is for callers
 * that must not call cudaMalloc while they run -- a controller evaluating
 * its policy inside a real-time loop, where an allocation can stall on
 * device-wide synchronisation, or a process whose device memory belongs to
 * another framework's pool. d_Gamma [r][n], d_pi [r] and d_b [n] are device
 * pointers; *Vb and *a are host results (FP64 value, action of the
 * maximising alpha, lowest index on ties, as pomdp_pbvi_value_gpu). The call
 * allocates nothing: its scratch is a fixed device array of
 * NOVA_VALUE_NOALLOC_MAX_ROWS doubles that every GPU loading the library
 * keeps until exit; r beyond that limit is rejected with
 * NOVA_ERROR_INVALID_DATA. Calls share the scratch, so calls that overlap on
 * the GPU race and must be serialised by the caller. The first call on a
 * device resolves the scratch's device address for it (again after the
 * device's context is created anew, e.g. after cudaDeviceReset); make that
 * first call before any stream capture. Kernels run on the calling thread's
 * per-thread default stream, which is not ordered against the caller's
 * non-blocking streams or other host threads: work that writes d_Gamma, d_pi
 * or d_b there must be complete before the call. The call returns after the
 * result is copied back. */
#define NOVA_VALUE_NOALLOC_MAX_ROWS 65536u
NOVA_API int pomdp_alpha_vectors_value_noalloc_gpu(const float *d_Gamma, const unsigned int *d_pi,
        unsigned int r, unsigned int n, const float *d_b, double *Vb, unsigned int *a);

/* Number of kernels this library has launched since it was loaded. */
NOVA_API unsigned long long nova_gb300_kernel_launches(void);

/* Test hook: make the count-th future call of a CUDA wrapper of the given
 * kind fail on the host, without calling CUDA (kind 1 = device allocation,
 * 2 = host-to-device copy, 3 = device-to-host copy, 4 = kernel launch).
 * count 0 disarms it. */
NOVA_API void nova_gb300_inject_fault(unsigned int kind, unsigned int count);

NOVA_NS_END

#endif
