// nova-gb300 internal: the point-based backup engine shared by PBVI and
// Perseus (device buffers, step-invariant tables, per-step scratch) and the
// interface between the exact-order kernels (pbvi.cu) and the tensor-core
// scoring path (pbvi_tc.cu).
#pragma once

#include "common.h"

#include <shared_mutex>

#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_gpu.h>
#include <nova/nova_gb300.h>

namespace nova_gb300 {

using nova::NovaPBVIStats;

// Device view of a POMDP model. All arrays are device pointers with the
// reference layouts: S,T [n][m][ns]; O [m][n][z]; R [n][m]; Z,B [r][rz].
struct DevModel {
    unsigned n, ns, m, z, r, rz;
    float gamma;
    const int *S;
    const float *T;
    const float *O;
    const float *R;
    const int *Z;
    const float *B;
};

struct TcState;  // tensor-core scoring state (pbvi_tc.cu)

// Addressing of the projection table: the value for (a*z+o, s, u) is
// base[ao * slice + s * sStride + u * uStride]. Two layouts are used:
// alpha-contiguous rows [m][z][n][uCols] (sStride = uCols, uStride = 1),
// read row-wise by the exact scan, and state-contiguous columns
// [m][z][uRows][sCols] (sStride = 1, uStride = sCols), read column-wise by
// the assembly of the chosen alphas.
struct ProjView {
    const float *base;
    size_t slice, sStride, uStride;
    __host__ __device__ __forceinline__ const float *slab(unsigned ao) const { return base + (size_t)ao * slice; }
    __host__ __device__ __forceinline__ size_t at(unsigned s, unsigned u) const { return s * sStride + u * uStride; }
};

// Exact-order kernel workspace and tables.
struct BackupEngine {
    DevModel md{};
    // Step-invariant tables (built once per model):
    unsigned *succLen = nullptr;   // [n*m]  successors before the first negative entry of row (s,a)
    unsigned *suppLen = nullptr;   // [r]    support entries before the first negative state of belief i
    float *C1 = nullptr;           // [m][n][ns][z]  fl(O[a,S(s,a,l),o] * T[s,a,l]); 0 past the row end
    float *C3 = nullptr;           // [m][z][n][ns]  same values, successor-contiguous
    // Per-step scratch:
    unsigned long long *hash = nullptr;  // [r] row hash of the input Gamma
    unsigned *rep = nullptr;             // [r] lowest index with a bitwise-identical row
    unsigned *uniqJ = nullptr;           // [r] unique index -> lowest original index
    unsigned *nUniqueDev = nullptr;      // device scalar
    float *Gt = nullptr;                 // [n][gtCols] transposed unique alphas
    size_t gtCols = 0;
    unsigned *jstar = nullptr;           // [r][m][z] chosen alpha per (belief, action, observation)
    unsigned *ustar = nullptr;           // [r][m][z] the same choice as a unique-alpha index
    float *Proj = nullptr;               // exact projections of the unique alphas (layout: ProjView)
    size_t projCap = 0, projCols = 0;    // projCols: alpha columns (rows in the state-contiguous layout)
    bool projStateMajor = false;         // this update's table is state-contiguous
    size_t projSCols = 0;                // states per column in the state-contiguous layout (n rounded to 8)
    bool projUnavailable = false, useProjNow = false;
    bool tableNever = false;             // NOVA_PBVI_TABLE_NEVER: no projection table, ever
    float *scanV = nullptr;              // running best of the chunked row scan
    unsigned *scanU = nullptr;
    size_t scanCap = 0;
    float *actVal = nullptr;             // [r][m] value of each action's assembled alpha at the belief
    float *partV = nullptr;              // [items][z][splits] split-scan partial maxima
    unsigned *partU = nullptr;
    size_t partCap = 0;
    unsigned *items = nullptr;           // [r*m] work list (belief*m + action)
    unsigned *itemCount = nullptr;       // device scalar
    unsigned *keptCount = nullptr;       // device scalar (count_kept)
    double *dotScratch = nullptr;        // [r] FP64 V(b) row values
    float *bDense = nullptr;             // [n]
    unsigned *resultA = nullptr;         // [1]
    double *resultV = nullptr;           // [1]
    float *rowScratch = nullptr;         // [n] single-belief alpha (Perseus)
    float *vnb = nullptr, *vnp1b = nullptr;  // [r] Perseus values over V_n and V_{n+1}
    unsigned *btilde = nullptr;          // [r] Perseus compacted belief list
    cudaStream_t stream = 0;
    cudaEvent_t ev[8] = {};
    bool eventsMade = false;
    unsigned scoring = NOVA_SCORING_FP16;
    NovaPBVIStats stats{};
    TcState *tc = nullptr;
    bool tcUnavailable = false;   // tensor-core operands could not be built (memory)
    static constexpr unsigned kTcMinUnique = 32;

    ~BackupEngine();
    int build(const DevModel &model, const char *fn);
    // One backup of every belief (PBVI): Gamma rows [0, rGamma) -> dst, pi.
    int backup_all(const float *src, unsigned rGamma, float *dst, unsigned *pi, const char *fn);
    // Dedup of Gamma rows [0, rows); returns the number of unique rows.
    int dedup(const float *src, unsigned rows, unsigned *nUnique, const char *fn);
    // Exact scoring of the listed (belief, action) items over the unique rows.
    int exact_score(const unsigned *items, unsigned nItems, unsigned nU, const char *fn);
    // Without the table: exact scoring of the (belief, action) items of the
    // listed (a*z+o)*r + i rows (count on the device in itemCount).
    int scan_rows_direct(const unsigned *rowList, unsigned nRows, unsigned nU, const char *fn);
    // Projection table for nU unique alphas (false if it does not fit).
    bool ensure_proj(unsigned nU);
    int project(unsigned nU, const char *fn);
    ProjView proj_view() const {
        if (projStateMajor) return ProjView{Proj, projCols * projSCols, 1, projSCols};
        return ProjView{Proj, (size_t)md.n * projCols, projCols, 1};
    }
    // Exact scan of (a*z+o)*r + i rows over the projection table (all rows if rowList is null).
    // With nRowsDev the row count is read on the device (nRows is then its upper bound).
    int scan_rows(const unsigned *rowList, unsigned nRows, unsigned nU, const char *fn,
                  const unsigned *nRowsDev = nullptr);
    // One update without host read-backs, for graph capture: every alpha
    // is scored as its own (uniqJ must be the identity), tensor-core
    // scoring with the solver's fixed schedule, the exact scan sized on the
    // device. Same results as backup_all.
    int backup_fixed(const float *src, float *dst, unsigned *pi, const char *fn);
    // backup_fixed in two halves around the scoring GEMM (tensor) or, with
    // tensor false, an update that scans every row exactly; no host
    // read-back in either.
    int fixed_pre(const float *src, bool tensor, const char *fn);
    int fixed_post(const float *src, float *dst, unsigned *pi, bool tensor, const char *fn);
    // Identity unique-alpha map and exact-scan capacity for every row, which
    // the fixed updates need.
    int fixed_setup(const char *fn);
    // Ready for backup_fixed: tensor-core scoring built with a fixed
    // schedule, the projection table allocated for all r alphas.
    bool fixed_ready() const;
    // Graphs of backup_fixed, one per direction (Gamma -> GammaPrime and back).
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    const float *graphSrc[2] = {nullptr, nullptr};
    unsigned graphLaunches[2] = {0, 0};
    bool graphMode = false;
    bool identityUniq = false;     // uniqJ holds 0 .. r-1
    bool capturing = false;        // launches are being captured, not run
    bool projAttrDone = false;     // shared-memory attributes of the projection kernels set
    float lastScanFrac = 0.0f;     // share of rows the last tensor-core update left to the exact scan
    bool state_major_wanted(size_t smemSM) const;
    // Work list of `count` consecutive items starting at `first`.
    int fill_items(unsigned first, unsigned count, const char *fn);
    // Write the last backup's selections (action per belief, alpha per
    // (belief, observation) under that action) to device arrays.
    int record(const unsigned *pi, unsigned *actOut, unsigned *selOut, const char *fn);
    // Action values and best-action assembly for all beliefs (or one).
    int assemble(const float *src, float *dst, unsigned *pi, int onlyBelief, float *dstRowOverride,
                 unsigned *actionOut, const char *fn);
    // After backup_all: the number of beliefs whose every action value
    // failed to beat the -1e10 sentinel (their row and action were left as
    // they were in dst and pi).
    int count_kept(unsigned *out, const char *fn);
};

// Held exclusively while an update graph is captured, shared by everything
// else that may run beside a capture in another host thread.
std::shared_mutex &capture_lock();

// The backup engine of an initialized device solver whose tables are built
// (after its first update), or null.
BackupEngine *pbvi_gpu_engine(const nova::POMDPPBVIGPU *pbvi);

// Tensor-core scoring (pbvi_tc.cu). tc_supported: the shapes fit the GEMM.
bool tc_supported(const DevModel &md);
// Builds the BF16 operand tables once; returns NOVA_SUCCESS or an error.
int tc_build(BackupEngine &eng, const char *fn);
// Scores every (belief, action, observation) row against the nU unique rows
// of src (gathered through eng.uniqJ), writes eng.jstar for rows whose argmax
// is proven, and appends the (belief, action) items that need the exact full
// scan to *rowList / *nRows as (a*z+o)*r + i row indices (a device list
// owned by the tensor-core state, sized for every row).
// The launches of tc_score without its read-back: the flagged rows and their
// count stay on the device (eng.tc rowList, eng.itemCount); `timed` records
// the GEMM events.
int tc_score_launch(BackupEngine &eng, const float *src, unsigned nU, bool timed, const char *fn);
// The three parts of tc_score_launch: packing, margins and schedule (kept in
// the state for the other two), the GEMM of this solver alone, and the
// merge with the exact-scan list.
int tc_prepare(BackupEngine &eng, const float *src, unsigned nU, const char *fn);
int tc_gemm(BackupEngine &eng, bool timed, const char *fn);
int tc_finish(BackupEngine &eng, const char *fn);
// The distinct (belief, action) items of the listed rows into eng.items
// (count in eng.itemCount, on the device).
int tc_rows_to_items(BackupEngine &eng, const unsigned *rowList, unsigned nRows, const char *fn);
// One persistent scoring launch (per candidate-list length) over the work
// units of many prepared solvers, drawn from a device table of their
// tensor maps, shapes and candidate arrays; the table is built once from
// the solvers' prepared launches and stays valid while their schedules,
// operands and alpha counts do.
struct TcBatch;
int tc_batch_create(BackupEngine *const *engs, unsigned count, TcBatch **out, const char *fn);
int tc_batch_gemm(TcBatch *batch, cudaStream_t stream, const char *fn);
void tc_batch_release(TcBatch *batch);
bool tc_schedule_fixed(const BackupEngine &eng);  // and built for eng.scoring
const unsigned *tc_row_list(const BackupEngine &eng);
int tc_score(BackupEngine &eng, const float *src, unsigned nU, unsigned *nRows, const unsigned **rowList,
             const char *fn);
void tc_release(TcState *tc);
// Per-belief detail of the last tensor-core update: alphas re-scored exactly
// and rows sent to the exact scan, summed over the belief's (a, o) rows.
int tc_row_detail(const BackupEngine &eng, unsigned *candidates, unsigned *exactRows, const char *fn);
// Feeds one tensor-core update's scoring time (GEMM, merge and the exact
// scan it left) to the solver's alpha-group tuner.
void tc_tune_feedback(BackupEngine &eng, float msScoring, unsigned nU);
// Scoring time per unique alpha of the tuned schedule (ms), or a negative
// value when the schedule was fixed without timing.
float tc_tuned_cost(const BackupEngine &eng);
unsigned tc_device_error();

}  // namespace nova_gb300
