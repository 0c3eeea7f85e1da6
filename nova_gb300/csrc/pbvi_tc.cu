// nova-gb300: tensor-core belief scoring for the point-based backup.
//
// The score of alpha j for (belief i, action a, observation o) is
//     score = sum_k B[i,k] * gamma * sum_l O(a,S,o) T(s_k,a,l) Gamma_j(S)
//           = sum_s A_ao[i,s] * Gamma_j[s],
//     A_ao[i,s] = gamma * O(a,s,o) * sum_{k,l : S(s_k,a,l) = s} B[i,k] T(s_k,a,l),
// a dense (r x n) . (n x |Gamma|) product per (a,o) pair. A_ao does not
// depend on Gamma: it is built once in FP16 or BF16 ([m*z][rPad][nPad],
// K-major, each row scaled by a power of two). Each update packs the unique
// alphas, shifted by a per-state midpoint c[s] (which changes every score of
// a row by the same amount), into FP16 -- or, for BF16, into a pair of BF16
// terms hi + lo whose sum carries 16 bits -- and the GEMM scores every row
// against every unique alpha on the tcgen05 tensor cores with FP32
// accumulation in TMEM. The epilogue keeps, per row, the best (score, alpha)
// pairs of each list and the best score it dropped; the scores never reach
// HBM.
//
// Exactness: for every row the kernel's score differs from the reference's
// FP32 score (pomdp_pbvi_cpu.cpp:50-83) by at most
//     E = a1 * (U * gmax + g_N * Gmax) + d1 * gmax
// (a1 = sum_s |A_ao[i,s]|, d1 = sum_s |A_ao[i,s] - half(A_ao[i,s])| the row's
// measured operand rounding, gmax = max |Gamma - c|, Gmax = max |Gamma|; U
// covers the rounding of the alphas, the FP32 build of A and the tensor-core
// accumulation; g_N = (ns + rz + 3) * 2^-24 covers the reference's own
// rounding). Every alpha within 2E of the best is re-scored in the
// reference's exact FP32 order and the argmax taken there; if the
// dropped-score bound says a candidate may be missing, the (belief, action)
// pair is rescanned exactly over all alphas. The chosen alphas are therefore
// exactly the reference's.
//
// GEMM kernel: persistent, one CTA per SM, 10 warps: warp 0 issues TMA loads
// (SWIZZLE_128B tiles 128x64 of A and 256x64 of the alphas into a 4-stage
// ring; with split alphas each A tile is loaded for the hi and then for the
// lo block), warp 1 issues tcgen05.mma (M=128, N=256, K=16, cta_group::1) into
// two 256-column TMEM accumulators, warps 2-9 drain TMEM with tcgen05.ld
// (two warps per lane quarter, alternate 32-column chunks) and run the top-8
// epilogue, skipping scores that lie below the row's margin under the
// running best, while the next tile accumulates. Work units are
// (a*z+o, 128-row tile, alpha group); units that run concurrently share
// their A tile and stream the same alphas, so both stay in L2. Every
// mbarrier wait is bounded; on timeout the kernel records an error word,
// stops issuing, frees its TMEM and returns.

#include "pbvi.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>
#include <cmath>

namespace nova_gb300 {

__device__ unsigned int g_device_error = 0;

unsigned read_and_clear_device_error() {
    unsigned h = 0;
    if (cudaMemcpyFromSymbol(&h, g_device_error, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (h != 0) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_device_error, &zero, sizeof(unsigned));
    }
    return h;
}

unsigned tc_device_error() { return read_and_clear_device_error(); }

constexpr int BM = 128;            // rows (beliefs) per tile
constexpr int BN = 256;            // alphas per tile
constexpr int BK = 64;             // K (states) per stage: 128 bytes of BF16
constexpr int STAGES = 4;
constexpr int MAX_TOPK = 32;       // entries per candidate list (layout capacity)
constexpr int MAX_LISTS = 8;       // candidate lists per row: two per alpha group
constexpr int MAX_ENTRIES = MAX_LISTS * MAX_TOPK;
constexpr int kLaneEntries = MAX_ENTRIES / 32;   // list entries per lane in the merge
constexpr unsigned kNoneU = 0xffffffffu;
constexpr int A_STAGE_BYTES = BM * BK * 2;   // 16 KB
constexpr int B_STAGE_BYTES = BN * BK * 2;   // 32 KB
constexpr int EPI_WARPS = 8;          // two per TMEM lane quarter
constexpr int GEMM_THREADS = 64 + 32 * EPI_WARPS;
constexpr size_t GEMM_SMEM = (size_t)STAGES * (A_STAGE_BYTES + B_STAGE_BYTES) + 1024 + 256;
constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz

struct TcState {
    size_t nPad = 0, rPad = 0, capN = 0;
    unsigned MZ = 0, mTiles = 0;
    unsigned mode = 0;              // NOVA_SCORING_BF16 or NOVA_SCORING_FP16: element type of A and Gb
    const float *src = nullptr;     // alpha set of the last prepared launch (rows of n)
    uint16_t *A = nullptr;          // [MZ][rPad][nPad] BF16 or FP16 bits, each row scaled by a power of 2
    float *a1 = nullptr;            // [MZ][rPad] bound of sum_s |A| in the row's scaled units
    float *a1raw = nullptr;         // [MZ][rPad] the same bound unscaled
    float *d1 = nullptr;            // [MZ][rPad] sum_s |A - half(A)| (scaled units): A's actual operand rounding
    uint16_t *Gb = nullptr;         // [capN][nPad] FP16, or [capN][2 nPad] split BF16, bits of (alpha - c) * 2^gexp
    float *shift = nullptr;         // [n]
    unsigned *scal = nullptr;       // [0] gmax, [1] Gmax, [2] escale, [3..4] counters, [5] max half-range, [6] G scale, [7] dscale (float bits)
    float *candV = nullptr;         // [MZ][r][MAX_LISTS][MAX_TOPK] (the first K entries of each list used)
    unsigned *candU = nullptr;
    float *candX = nullptr;         // [MZ][r][MAX_LISTS]
    unsigned *rowFlag = nullptr;    // [MZ*r] rows needing the exact scan
    unsigned *rowCand = nullptr;    // [MZ*r] alphas each row re-scored exactly in the merge
    unsigned *rowList = nullptr;    // [MZ*r] their indices, compacted
    unsigned *chunkCount = nullptr; // [ceil(MZ*r / 4096)] flagged rows per chunk, then chunk offsets
    unsigned *badModel = nullptr;   // [1] set when a probability is negative or NaN
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    CUtensorMap tmA;
    cudaEvent_t g0 = nullptr, g1 = nullptr;
    int numSMs = 0;
    // Scoring schedule: alpha groups per row tile and entries per candidate
    // list. Fewer groups and shorter lists make the epilogue cheaper; more
    // room in the lists leaves fewer rows to the exact scan. The best choice
    // depends on the shape, so each solver times kSchedules on its first
    // tensor-core updates (scoring plus the exact scan it leaves, per unique
    // alpha) and keeps the fastest. Results are identical for every choice.
    int schedFixed = -1;            // chosen schedule, -1 while tuning
    unsigned tuneNext = 0;          // next trial
    bool tuneWarm = false;          // the first tensor-core update (lazy set-up) is not timed
    unsigned groupsUsed = 0;        // groups of the last launch
    float tuneCost[3] = {0, 0, 0};  // one per tuned schedule
    // The launch prepared by tc_prepare for tc_gemm / tc_finish.
    struct Launch {
        unsigned nU = 0, nTiles = 0, groups = 0, lists = 0, topk = 0, kSplit = 1;
        bool fp16 = true;
        CUtensorMap tmB;
    } last;
};

// Schedules: alpha groups per row tile and entries per candidate list.
struct TcSchedule {
    unsigned groups, topk;
};
constexpr TcSchedule kSchedules[4] = {{4u, 16u}, {4u, 8u}, {2u, 8u}, {4u, 32u}};
constexpr int kTunedSchedules = 3;  // the first three are timed on small models
// Deep contractions use the most lists without tuning: FP16 with 16 entries
// per list; BF16, whose margin admits several times more candidates, 32.
constexpr int kDeepScheduleFp16 = 0, kDeepScheduleBf16 = 3;
// Deep contractions keep the epilogue hidden behind the MMAs; they use the
// most lists (best resolution) without tuning.
constexpr size_t kTuneMaxNPad = 2048;

void tc_release(TcState *tc) {
    if (!tc) return;
    cudaFree(tc->A); cudaFree(tc->a1); cudaFree(tc->a1raw); cudaFree(tc->d1); cudaFree(tc->Gb); cudaFree(tc->shift); cudaFree(tc->scal);
    cudaFree(tc->candV); cudaFree(tc->candU); cudaFree(tc->candX); cudaFree(tc->rowFlag); cudaFree(tc->rowCand); cudaFree(tc->rowList);
    cudaFree(tc->chunkCount);
    cudaFree(tc->badModel);
    if (tc->g0) cudaEventDestroy(tc->g0);
    if (tc->g1) cudaEventDestroy(tc->g1);
    delete tc;
}

bool tc_supported(const DevModel &md) {
    // The dense row of W_a must fit in shared memory while A is built, and
    // the row index must stay in TMA's 32-bit coordinate range.
    const size_t nPad = round_up(md.n, BK), rPad = round_up(md.r, BM);
    return md.n <= 40000 && (size_t)md.m * md.z * rPad < (1ull << 31) && nPad < (1ull << 31) && md.r >= 1;
}

// ---------------------------------------------------------------------------
// PTX wrappers (tcgen05 / TMA / mbarrier)
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (after recording a device error and raising
// the CTA's abort flag) if the phase does not complete in ~2 s, or if
// another role of the CTA already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abortFlag) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abortFlag) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abortFlag = 1;
            atomicExch(&g_device_error, 1u);
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor for a K-major, 128-byte-swizzled tile
// whose 8-row groups are 1024 bytes apart (the layout TMA writes with
// CU_TENSOR_MAP_SWIZZLE_128B and a 128-byte inner box).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;              // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;    // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1u << 46;              // descriptor version (tcgen05)
    d |= (uint64_t)2u << 61;              // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::f16: D FP32; A and B both BF16 (format 1) or
// both FP16 (format 0), K-major; M=128, N=256.
__host__ __device__ constexpr uint32_t make_idesc(uint32_t fmt) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}

// ---------------------------------------------------------------------------
// The scoring GEMM with the top-8 epilogue
// ---------------------------------------------------------------------------

struct GemmBarriers {
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    uint64_t accFull[2];
    uint64_t accEmpty[2];
    uint32_t tmemBase;
    int abortFlag;
};

__device__ __forceinline__ void decode_unit(unsigned unit, unsigned groups, unsigned mTiles, unsigned nTiles,
                                            unsigned &ao, unsigned &mt, unsigned &g, unsigned &nt0, unsigned &nt1) {
    g = unit % groups;
    const unsigned t = unit / groups;
    mt = t % mTiles;
    ao = t / mTiles;
    nt0 = (unsigned)((unsigned long long)g * nTiles / groups);
    nt1 = (unsigned)((unsigned long long)(g + 1) * nTiles / groups);
}

// Sorted top-K of (score, alpha) in registers; `excl` is the best score
// that fell off (or never entered) the list.
template <int K>
struct TopList {
    float v[K];
    unsigned u[K];
    float excl;
    __device__ __forceinline__ void reset() {
#pragma unroll
        for (int k = 0; k < K; k++) { v[k] = -INFINITY; u[k] = kNoneU; }
        excl = -INFINITY;
    }
    __device__ __forceinline__ void push(float x, unsigned idx) {
        if (!(x > v[K - 1])) {   // also drops NaN
            excl = fmaxf(excl, x);
            return;
        }
        excl = fmaxf(excl, v[K - 1]);
        // insertion from the bottom; equal scores keep the earlier (lower) index first
#pragma unroll
        for (int k = K - 1; k > 0; k--) {
            const bool shift = x > v[k - 1];
            const bool place = !shift && x > v[k];
            if (shift) { v[k] = v[k - 1]; u[k] = u[k - 1]; }
            else if (place) { v[k] = x; u[k] = idx; }
        }
        if (x > v[0]) { v[0] = x; u[0] = idx; }
    }
};

// Branch-free helpers over one 32-column chunk of a row's scores.
__device__ __forceinline__ float chunk_max(const float (&v)[32]) {
    float t[16];
#pragma unroll
    for (int k = 0; k < 16; k++) t[k] = fmaxf(v[2 * k], v[2 * k + 1]);
#pragma unroll
    for (int w = 8; w > 0; w >>= 1)
#pragma unroll
        for (int k = 0; k < w; k++) t[k] = fmaxf(t[2 * k], t[2 * k + 1]);
    return t[0];
}
__device__ __forceinline__ unsigned chunk_mask(const float (&v)[32], float lim) {
    unsigned t[16];
#pragma unroll
    for (int k = 0; k < 16; k++)
        t[k] = (v[2 * k] >= lim ? 1u << (2 * k) : 0u) | (v[2 * k + 1] >= lim ? 1u << (2 * k + 1) : 0u);
#pragma unroll
    for (int w = 8; w > 0; w >>= 1)
#pragma unroll
        for (int k = 0; k < w; k++) t[k] = t[2 * k] | t[2 * k + 1];
    return t[0];
}
// The smallest float above a finite or -inf f (+0 and -0 step to the
// smallest subnormal): x > f is x >= next_up(f) for every non-NaN x.
__device__ __forceinline__ float next_up(float f) {
    const unsigned b = __float_as_uint(f);
    if ((b & 0x7fffffffu) == 0u) return __uint_as_float(1u);
    return __uint_as_float((b & 0x80000000u) ? b - 1u : b + 1u);
}
// v[c] for a run-time c without indexing the register array.
__device__ __forceinline__ float chunk_select(const float (&v)[32], unsigned c) {
    float t[16];
#pragma unroll
    for (int k = 0; k < 16; k++) t[k] = (c & 1u) ? v[2 * k + 1] : v[2 * k];
    unsigned bit = 2u;
#pragma unroll
    for (int w = 8; w > 0; w >>= 1, bit <<= 1)
#pragma unroll
        for (int k = 0; k < w; k++) t[k] = (c & bit) ? t[2 * k + 1] : t[2 * k];
    return t[0];
}

// Twice the row's proven error bound (scaled units): the score gap within
// which an alpha may still be the exact argmax. The GEMM's filter and the
// merge's cut use this same expression.
__device__ __forceinline__ float row_margin(const float *__restrict__ a1, const float *__restrict__ d1, size_t idx,
                                            float escale, float dscale) {
    return 2.0f * (a1[idx] * escale + d1[idx] * dscale);
}

// What a work unit needs: its tensor maps, its place (a*z+o pair, 128-row
// tile, alpha group and the group's 256-alpha tiles) and its solver's shapes,
// bounds and candidate lists.
struct UnitParams {
    const CUtensorMap *tmA, *tmB;
    unsigned ao, mt, g, nt0, nt1;
    unsigned rPad, r, nU, kBlocks, kSplit;
    const float *a1, *d1;
    const unsigned *scal;
    float *candV;
    unsigned *candU;
    float *candX;
};

// One solver's units (the tensor maps are kernel parameters).
struct SingleUnits {
    unsigned MZ, rPad, r, mTiles, nTiles, groups, nU, kBlocks, kSplit;
    const float *a1, *d1;
    const unsigned *scal;
    float *candV;
    unsigned *candU;
    float *candX;
    __device__ __forceinline__ unsigned total() const { return MZ * mTiles * groups; }
    __device__ __forceinline__ void get(unsigned unit, UnitParams &p) const {
        decode_unit(unit, groups, mTiles, nTiles, p.ao, p.mt, p.g, p.nt0, p.nt1);
        p.rPad = rPad; p.r = r; p.nU = nU; p.kBlocks = kBlocks; p.kSplit = kSplit;
        p.a1 = a1; p.d1 = d1; p.scal = scal; p.candV = candV; p.candU = candU; p.candX = candX;
    }
};

// A solver of a batched launch: its tensor maps in global memory (aligned as
// CUtensorMap requires, which the struct inherits) and its first unit in the
// launch's unit sequence.
struct BatchModel {
    CUtensorMap tmA, tmB;
    unsigned unitStart, MZ, rPad, r, mTiles, nTiles, groups, nU, kBlocks, kSplit;
    const float *a1, *d1;
    const unsigned *scal;
    float *candV;
    unsigned *candU;
    float *candX;
};

// The units of many solvers in one sequence (solver k owns units
// [unitStart_k, unitStart_{k+1})): a device work table the persistent CTAs
// draw from.
struct BatchUnits {
    const BatchModel *models;
    unsigned nModels, totalUnits;
    __device__ __forceinline__ unsigned total() const { return totalUnits; }
    __device__ __forceinline__ void get(unsigned unit, UnitParams &p) const {
        unsigned lo = 0, hi = nModels - 1;
        while (lo < hi) {   // last model whose first unit is <= unit
            const unsigned mid = (lo + hi + 1) >> 1;
            if (models[mid].unitStart <= unit) lo = mid;
            else hi = mid - 1;
        }
        const BatchModel &b = models[lo];
        decode_unit(unit - b.unitStart, b.groups, b.mTiles, b.nTiles, p.ao, p.mt, p.g, p.nt0, p.nt1);
        p.tmA = &b.tmA; p.tmB = &b.tmB;
        p.rPad = b.rPad; p.r = b.r; p.nU = b.nU; p.kBlocks = b.kBlocks; p.kSplit = b.kSplit;
        p.a1 = b.a1; p.d1 = b.d1; p.scal = b.scal; p.candV = b.candV; p.candU = b.candU; p.candX = b.candX;
    }
};

template <int K, class Units>
__global__ void __launch_bounds__(GEMM_THREADS, 1) tc_score_gemm_kernel(
        const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, uint32_t idesc,
        const Units units) {
    extern __shared__ uint8_t smemRaw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;
    uint8_t *sB = smem + STAGES * A_STAGE_BYTES;
    GemmBarriers *bar = reinterpret_cast<GemmBarriers *>(smem + STAGES * (A_STAGE_BYTES + B_STAGE_BYTES));
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(smem_u32(&bar->full[s]), 1);
            mbar_init(smem_u32(&bar->empty[s]), 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(smem_u32(&bar->accFull[a]), 1);
            mbar_init(smem_u32(&bar->accEmpty[a]), EPI_WARPS);
        }
        bar->abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;"
                     ::"r"(smem_u32(&bar->tmemBase)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = bar->tmemBase;
    volatile int *abortFlag = &bar->abortFlag;
    const unsigned totalUnits = units.total();
    // Units of a single solver take the tensor maps from the kernel
    // parameters; a batch's from its work table.
    auto unit_params = [&](unsigned unit, UnitParams &p) {
        units.get(unit, p);
        if constexpr (std::is_same<Units, SingleUnits>::value) { p.tmA = &tmA; p.tmB = &tmB; }
    };

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            unsigned stage = 0, phase = 0;
            for (unsigned unit = blockIdx.x; unit < totalUnits && !*abortFlag; unit += gridDim.x) {
                UnitParams p;
                unit_params(unit, p);
                const int rowA = (int)(p.ao * p.rPad + p.mt * BM);
                for (unsigned nt = p.nt0; nt < p.nt1 && !*abortFlag; nt++) {
                    // kSplit B blocks per A block: the split alphas carry a hi
                    // and a lo block for each 64-state block of A.
                    for (unsigned kb = 0; kb < p.kBlocks * p.kSplit; kb++) {
                        if (!mbar_wait(smem_u32(&bar->empty[stage]), phase ^ 1u, abortFlag)) break;
                        const uint32_t fb = smem_u32(&bar->full[stage]);
                        mbar_expect_tx(fb, A_STAGE_BYTES + B_STAGE_BYTES);
                        tma_load_2d(smem_u32(sA + stage * A_STAGE_BYTES), p.tmA, (int)((kb / p.kSplit) * BK), rowA, fb);
                        tma_load_2d(smem_u32(sB + stage * B_STAGE_BYTES), p.tmB, (int)(kb * BK), (int)(nt * BN), fb);
                        if (++stage == STAGES) { stage = 0; phase ^= 1u; }
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            unsigned stage = 0, phase = 0, acc = 0, accPhase = 0;
            for (unsigned unit = blockIdx.x; unit < totalUnits && !*abortFlag; unit += gridDim.x) {
                UnitParams p;
                unit_params(unit, p);
                for (unsigned nt = p.nt0; nt < p.nt1 && !*abortFlag; nt++) {
                    if (!mbar_wait(smem_u32(&bar->accEmpty[acc]), accPhase ^ 1u, abortFlag)) break;
                    tc_fence_after();
                    const uint32_t dtmem = tmem + acc * BN;
                    for (unsigned kb = 0; kb < p.kBlocks * p.kSplit; kb++) {
                        if (!mbar_wait(smem_u32(&bar->full[stage]), phase, abortFlag)) break;
                        tc_fence_after();
                        const uint64_t adesc = smem_desc_sw128(smem_u32(sA + stage * A_STAGE_BYTES));
                        const uint64_t bdesc = smem_desc_sw128(smem_u32(sB + stage * B_STAGE_BYTES));
#pragma unroll
                        for (int kk = 0; kk < BK / 16; kk++)
                            umma_f16(dtmem, adesc + 2u * kk, bdesc + 2u * kk, idesc,
                                     (kb | (unsigned)kk) != 0u ? 1u : 0u);
                        umma_commit(smem_u32(&bar->empty[stage]));
                        if (++stage == STAGES) { stage = 0; phase ^= 1u; }
                    }
                    umma_commit(smem_u32(&bar->accFull[acc]));
                    acc ^= 1u;
                    if (acc == 0) accPhase ^= 1u;
                }
            }
        }
    } else {
        // ---- epilogue: TMEM -> registers -> running top-8 per row ----
        // Eight warps: warps w and w+4 read the same TMEM lane quarter
        // (w & 3), one row per thread, and take alternate 32-column chunks
        // of every tile, each keeping its own list for the unit (list
        // 2g + half of the row).
        // A score below (running best - thr), thr being the row's margin as
        // the merge computes it, lies below the merge's cut for every later
        // best (the cut is fl(final best - thr) and rounding is monotonic):
        // it can be neither a candidate nor the dropped score that sends the
        // row to the exact scan, so it is skipped without touching the list.
        // A chunk whose maximum is below the limit costs a few branch-free
        // instructions; otherwise the limit is raised to the chunk's maximum
        // minus thr and only the chunk's scores at or above it go through
        // the list, one set bit of the chunk's mask at a time.
        const unsigned quarter = warp & 3u;   // TMEM lanes this warp may access
        const unsigned half = (warp - 2u) >> 2;
        const unsigned rowInTile = quarter * 32u + lane;
        const float qnan = __uint_as_float(0x7fc00000u);
        unsigned acc = 0, accPhase = 0;
        TopList<K> top;
        for (unsigned unit = blockIdx.x; unit < totalUnits && !*abortFlag; unit += gridDim.x) {
            UnitParams p;
            unit_params(unit, p);
            const unsigned ao = p.ao, g = p.g, r = p.r, nU = p.nU;
            const float escale = __uint_as_float(p.scal[2]);
            const float dscale = __uint_as_float(p.scal[7]);
            top.reset();
            const unsigned iRow = p.mt * BM + rowInTile;
            // Same expression as the merge's margin. An infinite margin skips
            // nothing; a NaN one skips everything, and the merge sends such
            // rows to the exact scan whatever their lists hold.
            const float thr = iRow < r ? row_margin(p.a1, p.d1, (size_t)ao * p.rPad + iRow, escale, dscale) : INFINITY;
            float best = -INFINITY, lim = -INFINITY;
            bool ok = true;
            for (unsigned nt = p.nt0; nt < p.nt1; nt++) {
                if (!mbar_wait(smem_u32(&bar->accFull[acc]), accPhase, abortFlag)) { ok = false; break; }
                tc_fence_after();
                const uint32_t base = tmem + ((quarter * 32u) << 16) + acc * BN;
#pragma unroll 1
                for (unsigned ch = half; ch < BN / 32; ch += 2) {
                    __syncwarp();
                    float v[32];
                    tmem_ld32(base + ch * 32u, v);
                    const unsigned u0 = nt * BN + ch * 32u;
                    if (u0 + 32u > nU) {   // columns past the unique alphas are skipped (NaN)
#pragma unroll
                        for (int c = 0; c < 32; c++)
                            if (u0 + c >= nU) v[c] = qnan;
                    }
                    const float mx = chunk_max(v);
                    if (mx >= lim) {
                        // The chunk's maximum raises the running best first,
                        // so only its scores within thr of the new best are
                        // listed (the list's first entry is that best).
                        best = fmaxf(best, mx);
                        lim = best - thr;
                        // Scores at or below the list's last entry f would
                        // only raise the dropped maximum (push's first
                        // branch). If any score of the chunk is above f, its
                        // insertion drops f itself, which bounds them all;
                        // otherwise the chunk's maximum is the largest of
                        // them. Either way the list and the dropped maximum
                        // end as if every score >= lim had been pushed.
                        unsigned mask = chunk_mask(v, fmaxf(lim, next_up(top.v[K - 1])));
                        if (mask == 0u) top.excl = fmaxf(top.excl, mx);
                        while (mask) {
                            const unsigned c = __ffs(mask) - 1;
                            mask &= mask - 1;
                            top.push(chunk_select(v, c), u0 + c);
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bar->accEmpty[acc]));
                acc ^= 1u;
                if (acc == 0) accPhase ^= 1u;
            }
            if (!ok) break;
            if (iRow < r) {
                const size_t slot = ((size_t)ao * r + iRow) * MAX_LISTS + 2u * g + half;
                float *cv = p.candV + slot * MAX_TOPK;
                unsigned *cu = p.candU + slot * MAX_TOPK;
#pragma unroll
                for (int k = 0; k < K; k++) { cv[k] = top.v[k]; cu[k] = top.u[k]; }
                p.candX[slot] = top.excl;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
}

// ---------------------------------------------------------------------------
// Step-invariant operand: A_ao[i, s] in BF16/FP16, each row scaled by a power
// of two so its largest entry lies in [2^13, 2^14) (FP16's precision is then
// used fully and nothing overflows); a1 bounds sum_s |A| in the same units.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint16_t to_half_bits(float v, bool fp16) {
    if (fp16) return __half_as_ushort(__float2half_rn(v));
    return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}
__device__ __forceinline__ float from_half_bits(uint16_t b, bool fp16) {
    if (fp16) return __half2float(__ushort_as_half(b));
    return __bfloat162float(__ushort_as_bfloat16(b));
}

__global__ void tc_build_a_kernel(DevModel md, const unsigned *__restrict__ succLen,
                                  const unsigned *__restrict__ suppLen, size_t rPad, size_t nPad, int fp16,
                                  uint16_t *__restrict__ A, float *__restrict__ a1, float *__restrict__ a1raw,
                                  float *__restrict__ d1, float a1Slack, float d1Slack,
                                  unsigned *__restrict__ badModel) {
    extern __shared__ float W[];  // [n]
    const unsigned i = blockIdx.x / md.m, a = blockIdx.x % md.m;
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) W[s] = 0.0f;
    __syncthreads();
    const unsigned Li = suppLen[i];
    for (unsigned e = threadIdx.x; e < Li * md.ns; e += blockDim.x) {
        const unsigned k = e / md.ns, l = e % md.ns;
        const int s = md.Z[(size_t)i * md.rz + k];
        if (l < succLen[(size_t)s * md.m + a]) {
            const size_t row = ((size_t)s * md.m + a) * md.ns + l;
            const float w = md.B[(size_t)i * md.rz + k] * md.T[row];
            if (!(w >= 0.0f)) atomicOr(badModel, 1u);  // the bound assumes non-negative B, T, O
            atomicAdd(&W[md.S[row]], w);
        }
    }
    __syncthreads();
    __shared__ float red[32], redD[32];
    __shared__ float rowScale;
    for (unsigned o = 0; o < md.z; o++) {
        const size_t ao = (size_t)a * md.z + o;
        uint16_t *row = A + (ao * rPad + i) * nPad;
        float mx = 0.0f, sum = 0.0f;
        for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
            const float ob = md.O[((size_t)a * md.n + s) * md.z + o];
            if (!(ob >= 0.0f)) atomicOr(badModel, 1u);
            const float v = md.gamma * W[s] * ob;
            mx = fmaxf(mx, v);
            sum += v;
        }
        for (int off = 16; off > 0; off >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
            sum += __shfl_xor_sync(0xffffffffu, sum, off);
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (unsigned w = 0; w < blockDim.x / 32; w++) mx = fmaxf(mx, red[w]);
            int e = 0;
            if (mx > 0.0f) frexpf(mx, &e);          // mx in [2^(e-1), 2^e)
            rowScale = mx > 0.0f ? ldexpf(1.0f, 14 - e) : 1.0f;
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
        __syncthreads();
        const float scale = rowScale;
        // d1 = sum_s |A - half(A)| in the row's scaled units: the actual
        // rounding of this row's operand (each term is exact in FP32).
        float dsum = 0.0f;
        for (unsigned s = threadIdx.x; s < nPad; s += blockDim.x) {
            float v = 0.0f;
            if (s < md.n) v = md.gamma * W[s] * md.O[((size_t)a * md.n + s) * md.z + o];
            const float x = v * scale;
            const uint16_t hb = to_half_bits(x, fp16 != 0);
            row[s] = hb;
            dsum += fabsf(x - from_half_bits(hb, fp16 != 0));
        }
        for (int off = 16; off > 0; off >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, off);
        if ((threadIdx.x & 31) == 0) redD[threadIdx.x >> 5] = dsum;
        __syncthreads();
        if (threadIdx.x == 0) {
            float t = 0.0f, d = 0.0f;
            for (unsigned w = 0; w < blockDim.x / 32; w++) { t += red[w]; d += redD[w]; }
            a1[ao * rPad + i] = t * scale * a1Slack;
            a1raw[ao * rPad + i] = t * a1Slack;
            d1[ao * rPad + i] = d * d1Slack;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Per-update packing of the unique alphas
// ---------------------------------------------------------------------------

__device__ __forceinline__ void atomic_max_nonneg(unsigned *addr, float v) {
    // Non-negative floats order like their bit patterns; NaN (all exponent
    // bits set, nonzero mantissa) compares above every finite value, which
    // disables the margin.
    atomicMax(addr, __float_as_uint(v));
}

// Per-state midpoint shift c[s] over the unique alphas, Gmax = max |alpha|
// (scal[1]) and the largest half-range max (hi - lo) / 2 (scal[5]).
__global__ void tc_shift_kernel(const float *__restrict__ Gt, size_t gtCols, unsigned n, unsigned nU,
                                float *__restrict__ shift, unsigned *__restrict__ scal) {
    const unsigned s = blockIdx.x;
    const float *row = Gt + (size_t)s * gtCols;
    float mn = INFINITY, mx = -INFINITY;
    int nanSeen = 0;
    for (unsigned u = threadIdx.x; u < nU; u += blockDim.x) {
        const float v = row[u];
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
        nanSeen |= (v != v);
    }
    __shared__ float smn[32], smx[32];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    for (int off = 16; off > 0; off >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, off));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    }
    __syncthreads();
    if (nanSeen) snan = 1;
    if ((threadIdx.x & 31) == 0) { smn[threadIdx.x >> 5] = mn; smx[threadIdx.x >> 5] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 0; w < blockDim.x / 32; w++) { mn = fminf(mn, smn[w]); mx = fmaxf(mx, smx[w]); }
        shift[s] = 0.5f * mn + 0.5f * mx;
        const float nanf_ = __uint_as_float(0x7fc00000u);
        atomic_max_nonneg(&scal[1], snan ? nanf_ : fmaxf(fabsf(mn), fabsf(mx)));
        atomic_max_nonneg(&scal[5], snan ? nanf_ : 0.5f * (mx - mn));
    }
}

// Power-of-two scale for the packed alphas: the largest |alpha - c| lands
// in [2^13, 2^14) (half-range plus slack for the rounding of c).
__global__ void tc_gscale_kernel(unsigned *scal) {
    const float hr = __uint_as_float(scal[5]) * 1.001f + 1e-30f;
    int e = 0;
    frexpf(hr, &e);
    scal[6] = __float_as_uint(hr < 1e30f ? ldexpf(1.0f, 13 - e) : 1.0f);
}

// Gb[u] = half((alpha_u(s) - c[s]) * gscale); rows >= nU, states >= n are 0.
// Single form (FP16): one value per state, row length nPad. Split form
// (BF16): each value v is carried as hi = bf16(v) and lo = bf16(v - hi)
// (v - hi is exact in FP32), so |v - hi - lo| <= 2^-16 |v|; the row holds,
// for every 64-state block kb, the 64 hi values and then the 64 lo values
// (row length 2 nPad), and the GEMM multiplies one A block by both.
// Records gmax = max |(alpha - c) * gscale| over the FP32 values.
__global__ void tc_pack_kernel(const float *__restrict__ G, unsigned n, size_t nPad, const unsigned *__restrict__ uniqJ,
                               unsigned nU, const float *__restrict__ shift, int fp16, int split,
                               uint16_t *__restrict__ Gb, unsigned *__restrict__ scal) {
    const unsigned u = blockIdx.x;
    const float gscale = __uint_as_float(scal[6]);
    const size_t rowLen = split ? 2 * nPad : nPad;
    uint16_t *out = Gb + (size_t)u * rowLen;
    float m = 0.0f;
    int nanSeen = 0;
    if (u < nU) {
        const float *row = G + (size_t)uniqJ[u] * n;
        for (unsigned s = threadIdx.x; s < nPad; s += blockDim.x) {
            float v = 0.0f;
            if (s < n) {
                v = (row[s] - shift[s]) * gscale;
                m = fmaxf(m, fabsf(v));
                nanSeen |= (v != v);
            }
            if (split) {
                const uint16_t hi = to_half_bits(v, false);
                const uint16_t lo = to_half_bits(v - from_half_bits(hi, false), false);
                const size_t at = (size_t)(s / BK) * (2 * BK) + (s % BK);
                out[at] = hi;
                out[at + BK] = lo;
            } else {
                out[s] = to_half_bits(v, fp16 != 0);
            }
        }
    } else {
        for (size_t s = threadIdx.x; s < rowLen; s += blockDim.x) out[s] = 0;
    }
    __shared__ float red[32];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    __syncthreads();
    if (nanSeen) snan = 1;
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned w = 0; w < blockDim.x / 32; w++) m = fmaxf(m, red[w]);
        atomic_max_nonneg(&scal[0], snan ? __uint_as_float(0x7fc00000u) : m);
    }
}

// escale = U * gmax + gN * Gmax * gscale and dscale = gmax (1 + 2^-22), all
// in the packed units; the per-row bound is a1 * escale + d1 * dscale.
__global__ void tc_escale_kernel(unsigned *scal, float U, float gN) {
    const float gmax = __uint_as_float(scal[0]);
    const float Gmax = __uint_as_float(scal[1]);
    const float gscale = __uint_as_float(scal[6]);
    scal[2] = __float_as_uint(U * gmax + gN * Gmax * gscale);
    scal[7] = __float_as_uint(gmax * (1.0f + 2.4e-7f));
}

// ---------------------------------------------------------------------------
// Merge the per-group lists, apply the proven margin, re-score near ties
// exactly from the projection table. One warp per (a*z+o, belief) row; rows
// whose candidate set may be incomplete go to the exact row scan.
// ---------------------------------------------------------------------------

// score(u) = sum_k fl(Proj[s_k][u] * b_k) in support order
// (pomdp_pbvi_cpu.cpp:50-83). Eight table entries are fetched before their
// eight ordered additions, so the gathers overlap.
__device__ __forceinline__ float proj_row_score(const float *__restrict__ P, const ProjView &pv, unsigned u,
                                                const float *__restrict__ bk, const int *__restrict__ sk, unsigned Li) {
    float v = 0.0f;
    unsigned k = 0;
    for (; k + 8 <= Li; k += 8) {
        float pq[8];
#pragma unroll
        for (int q = 0; q < 8; q++) pq[q] = P[pv.at((unsigned)sk[k + q], u)];
#pragma unroll
        for (int q = 0; q < 8; q++) v = fadd(v, fmul(pq[q], bk[k + q]));
    }
    for (; k < Li; k++) v = fadd(v, fmul(P[pv.at((unsigned)sk[k], u)], bk[k]));
    return v;
}

// Without the projection table: the same exact scores straight from the
// model and the alpha rows, in the table's order: each support state's
// entry fl(gamma * sum_l C * alpha(S)) (proj_state_lanes_kernel; C3 holds the
// same products as C1, successor-contiguous), times b_k, summed in support
// order.
constexpr unsigned kDirectNs = 32;  // successors per state the direct re-score holds in registers

struct DirectScorer {
    const unsigned *succLen;
    const float *C3, *G;  // G: the update's alpha set, rows of n
    __device__ __forceinline__ float vt(const DevModel &md, unsigned a, unsigned o, unsigned s,
                                        const float *__restrict__ Gj) const {
        const unsigned Ls = __ldg(succLen + (size_t)s * md.m + a);
        const float *c = C3 + (((size_t)a * md.z + o) * md.n + s) * md.ns;
        const int *sp = md.S + ((size_t)s * md.m + a) * md.ns;
        float v = 0.0f;
        for (unsigned l = 0; l < Ls; l++) v = fadd(v, fmul(__ldg(c + l), __ldg(Gj + __ldg(sp + l))));
        return v;
    }
};

// One warp per row; returns (in every lane) the number of candidates it
// re-scored exactly, 0 when the row was settled without re-scoring or sent to
// the exact scan. The row's lists hold K entries each; entry e of the warp's
// view is entry e / nLists of list e % nLists, so the lists' leading entries
// (where the candidates are) spread over the lanes.
template <bool kDirect>
__device__ __forceinline__ unsigned merge_row(size_t row, unsigned lane, DevModel md,
                                              const unsigned *__restrict__ suppLen, const ProjView pv,
                                              const DirectScorer ds, float *scratch,
                                              const unsigned *__restrict__ uniqJ, unsigned nLists,
                                              unsigned K, size_t rPad, const float *__restrict__ a1,
                                              const float *__restrict__ d1,
                                              const float *__restrict__ a1raw, const unsigned *__restrict__ scal,
                                              const float *__restrict__ candV, const unsigned *__restrict__ candU,
                                              const float *__restrict__ candX, unsigned *__restrict__ ustar,
                                              unsigned *__restrict__ jstar, unsigned *__restrict__ rowFlag,
                                              const unsigned *__restrict__ badModel) {
    const unsigned ao = (unsigned)(row / md.r), i = (unsigned)(row % md.r);
    const unsigned a = ao / md.z, o = ao % md.z;
    const size_t base = row * MAX_ENTRIES;
    const unsigned nEnt = nLists * K;     // <= MAX_ENTRIES: each lane holds entries lane + 32 j, j < kLaneEntries
    float v[kLaneEntries];
    unsigned u[kLaneEntries];
    float tmax = -INFINITY;
#pragma unroll
    for (int j = 0; j < kLaneEntries; j++) {
        const unsigned e = lane + 32u * j;
        v[j] = -INFINITY;
        u[j] = kNoneU;
        if (e < nEnt) {
            const size_t idx = base + (size_t)(e % nLists) * MAX_TOPK + e / nLists;
            u[j] = candU[idx];
            if (u[j] != kNoneU) v[j] = candV[idx];
        }
        tmax = fmaxf(tmax, v[j]);
    }
    float x = lane < nLists ? candX[row * MAX_LISTS + lane] : -INFINITY;
    for (int off = 16; off > 0; off >>= 1) {
        tmax = fmaxf(tmax, __shfl_xor_sync(0xffffffffu, tmax, off));
        x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, off));
    }
    const float thr = row_margin(a1, d1, (size_t)ao * rPad + i, __uint_as_float(scal[2]), __uint_as_float(scal[7]));
    // Usable only with a finite margin, non-negative probabilities, and
    // scores far from the reference's -1e10 sentinel.
    const float Gmax = __uint_as_float(scal[1]);
    const bool usable = (thr < 1e30f) && (tmax > -INFINITY) && *badModel == 0u &&
                        (a1raw[(size_t)ao * rPad + i] * Gmax < 1e9f);
    const float cut = tmax - thr;
    if (!usable || x >= cut) {
        if (lane == 0) rowFlag[row] = 1u;
        return 0u;
    }
    bool c[kLaneEntries];
    unsigned count = 0, first = kNoneU;
#pragma unroll
    for (int j = 0; j < kLaneEntries; j++) {
        c[j] = u[j] != kNoneU && v[j] >= cut;
        const unsigned msk = __ballot_sync(0xffffffffu, c[j]);
        count += __popc(msk);
        if (first == kNoneU && msk) first = 32u * j + __ffs(msk) - 1;
    }
    const size_t js = ((size_t)i * md.m + a) * md.z + o;
    if (count == 1) {
        const unsigned src = first & 31u, jj = first >> 5;
        unsigned mine = u[0];
#pragma unroll
        for (int j = 1; j < kLaneEntries; j++)
            if (jj == (unsigned)j) mine = u[j];
        const unsigned uu = __shfl_sync(0xffffffffu, mine, src);
        if (lane == 0) { ustar[js] = uu; jstar[js] = uniqJ[uu]; }
        return 0u;
    }
    const unsigned Li = suppLen[i];
    const int *sk = md.Z + (size_t)i * md.rz;
    const float *bk = md.B + (size_t)i * md.rz;
    float best = -INFINITY;
    unsigned bu = kNoneU;
    if constexpr (!kDirect) {
        // Several candidates: each lane re-scores its own in the exact order.
        const float *P = pv.slab(ao);
#pragma unroll
        for (int j = 0; j < kLaneEntries; j++) {
            if (c[j]) {
                const float w = proj_row_score(P, pv, u[j], bk, sk, Li);
                if (bu == kNoneU || w > best || (w == best && u[j] < bu)) { best = w; bu = u[j]; }
            }
        }
    } else {
        // Without the table the warp scores its candidates together, up to
        // 32 at a time (candidate t held by lane t): for every 32 support
        // states, lane k computes state k's term for each candidate of the
        // batch into the warp's scratch (the gathers of one candidate stay
        // in one alpha row), then lane t adds candidate t's terms in support
        // order.
        unsigned myU = kNoneU, nb = 0;
        auto flush = [&]() {
            float total = 0.0f;
            for (unsigned k0 = 0; k0 < Li; k0 += 32u) {
                const unsigned k = k0 + lane;
                const bool kv = k < Li;
                const unsigned s = kv ? (unsigned)sk[k] : 0u;
                const float b = kv ? bk[k] : 0.0f;
                if (md.ns <= kDirectNs) {
                    // The state's coefficients and successors, loaded once for
                    // the whole batch.
                    const unsigned Ls = kv ? __ldg(ds.succLen + (size_t)s * md.m + a) : 0u;
                    const float *cp = ds.C3 + (((size_t)a * md.z + o) * md.n + s) * md.ns;
                    const int *spp = md.S + ((size_t)s * md.m + a) * md.ns;
                    float cc[kDirectNs];
                    int ss[kDirectNs];
#pragma unroll
                    for (unsigned l = 0; l < kDirectNs; l++) {
                        cc[l] = l < Ls ? __ldg(cp + l) : 0.0f;
                        ss[l] = l < Ls ? __ldg(spp + l) : 0;
                    }
                    // Two candidates at a time: their gathers are issued
                    // together, their sums are two independent chains.
                    for (unsigned t = 0; t < nb; t += 2) {
                        const unsigned t1 = t + 1 < nb ? t + 1 : t;
                        const unsigned u0 = __shfl_sync(0xffffffffu, myU, t);
                        const unsigned u1 = __shfl_sync(0xffffffffu, myU, t1);
                        const float *G0 = ds.G + (size_t)__ldg(uniqJ + u0) * md.n;
                        const float *G1 = ds.G + (size_t)__ldg(uniqJ + u1) * md.n;
                        float g0[kDirectNs], g1[kDirectNs];
#pragma unroll
                        for (unsigned l = 0; l < kDirectNs; l++) {
                            if (l < Ls) {
                                g0[l] = __ldg(G0 + ss[l]);
                                g1[l] = __ldg(G1 + ss[l]);
                            }
                        }
                        float v0 = 0.0f, v1 = 0.0f;
#pragma unroll
                        for (unsigned l = 0; l < kDirectNs; l++) {
                            if (l < Ls) {
                                v0 = fadd(v0, fmul(cc[l], g0[l]));
                                v1 = fadd(v1, fmul(cc[l], g1[l]));
                            }
                        }
                        scratch[t * 32u + lane] = kv ? fmul(fmul(v0, md.gamma), b) : 0.0f;
                        if (t1 != t) scratch[t1 * 32u + lane] = kv ? fmul(fmul(v1, md.gamma), b) : 0.0f;
                    }
                } else {
                    for (unsigned t = 0; t < nb; t++) {
                        const unsigned uu = __shfl_sync(0xffffffffu, myU, t);
                        float p = 0.0f;
                        if (kv) p = fmul(fmul(ds.vt(md, a, o, s, ds.G + (size_t)__ldg(uniqJ + uu) * md.n), md.gamma), b);
                        scratch[t * 32u + lane] = p;
                    }
                }
                __syncwarp();
                if (lane < nb) {
                    const unsigned cnt = min(32u, Li - k0);
                    for (unsigned q = 0; q < cnt; q++) total = fadd(total, scratch[lane * 32u + q]);
                }
                __syncwarp();
            }
            if (lane < nb && (bu == kNoneU || total > best || (total == best && myU < bu))) { best = total; bu = myU; }
            nb = 0;
        };
#pragma unroll
        for (int j = 0; j < kLaneEntries; j++) {
            unsigned msk = __ballot_sync(0xffffffffu, c[j]);
            while (msk) {
                const unsigned src = __ffs(msk) - 1;
                msk &= msk - 1;
                const unsigned uu = __shfl_sync(0xffffffffu, u[j], src);
                if (lane == nb) myU = uu;
                if (++nb == 32u) flush();
            }
        }
        if (nb) flush();
    }
    for (int off = 16; off > 0; off >>= 1) {
        const float b2 = __shfl_xor_sync(0xffffffffu, best, off);
        const unsigned u2 = __shfl_xor_sync(0xffffffffu, bu, off);
        if (u2 != kNoneU && (bu == kNoneU || b2 > best || (b2 == best && u2 < bu))) { best = b2; bu = u2; }
    }
    if (lane == 0) {
        if (!(best > -1e10f)) {
            rowFlag[row] = 1u;  // sentinel case: the exact scan applies the reference's rule
        } else {
            ustar[js] = bu;
            jstar[js] = uniqJ[bu];
        }
    }
    return count;
}

// Rows re-scored and candidates re-scored are counted per block in shared
// memory, then added to the global counters once per block.
template <bool kDirect>
__global__ void __launch_bounds__(256, kDirect ? 1 : 2) tc_merge_kernel(DevModel md, const unsigned *__restrict__ suppLen,
                                const ProjView pv, const DirectScorer ds, const unsigned *__restrict__ uniqJ,
                                unsigned nLists, unsigned K,
                                size_t rPad, const float *__restrict__ a1, const float *__restrict__ d1,
                                const float *__restrict__ a1raw, const unsigned *__restrict__ scal,
                                const float *__restrict__ candV, const unsigned *__restrict__ candU,
                                const float *__restrict__ candX, unsigned *__restrict__ ustar,
                                unsigned *__restrict__ jstar, unsigned *__restrict__ rowFlag,
                                unsigned *__restrict__ rowCand, unsigned *__restrict__ counters,
                                const unsigned *__restrict__ badModel) {
    __shared__ unsigned blockCount[2];
    extern __shared__ float mergeScratch[];  // direct form: [warps][32 candidates][32 states]
    if (threadIdx.x == 0) { blockCount[0] = 0u; blockCount[1] = 0u; }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const size_t rows = (size_t)md.m * md.z * md.r;
    unsigned rescored = 0;
    if (row < rows)
        rescored = merge_row<kDirect>(row, lane, md, suppLen, pv, ds, mergeScratch + (threadIdx.x >> 5) * 1024u,
                                      uniqJ, nLists, K, rPad, a1, d1, a1raw, scal, candV, candU, candX, ustar, jstar,
                                      rowFlag, badModel);
    if (lane == 0 && row < rows) rowCand[row] = rescored;
    if (lane == 0 && rescored) {
        atomicAdd(&blockCount[0], 1u);
        atomicAdd(&blockCount[1], rescored);
    }
    __syncthreads();
    if (threadIdx.x == 0 && blockCount[0]) {
        atomicAdd(&counters[0], blockCount[0]);
        atomicAdd(&counters[1], blockCount[1]);
    }
}

// List of flagged rows in increasing order, in three launches: flagged rows
// per chunk of 4096, a one-block scan of the chunk counts, then each chunk
// writes its rows at its offset.
constexpr unsigned kCompactChunk = 4096;  // rows per block (4 per thread)

__global__ void __launch_bounds__(1024) tc_compact_count_kernel(const unsigned *__restrict__ flag, unsigned count,
                                                                unsigned *__restrict__ chunkCount) {
    const unsigned base = blockIdx.x * kCompactChunk;
    unsigned c = 0;
    for (unsigned k = threadIdx.x; k < kCompactChunk; k += blockDim.x)
        if (base + k < count && flag[base + k]) c++;
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    __shared__ unsigned ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (unsigned w = 0; w < blockDim.x / 32; w++) t += ws[w];
        chunkCount[blockIdx.x] = t;
    }
}

// Exclusive scan of chunkCount[0..nChunks) in place; the total goes to *nOut.
__global__ void __launch_bounds__(1024) tc_compact_scan_kernel(unsigned *__restrict__ chunkCount, unsigned nChunks,
                                                               unsigned *__restrict__ nOut) {
    __shared__ unsigned sums[1024];
    const unsigned per = (nChunks + blockDim.x - 1) / blockDim.x;
    const unsigned b = threadIdx.x * per, e = min(nChunks, b + per);
    unsigned s = 0;
    for (unsigned i = b; i < e; i++) s += chunkCount[i];
    sums[threadIdx.x] = s;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
        const unsigned v = threadIdx.x >= off ? sums[threadIdx.x - off] : 0u;
        __syncthreads();
        sums[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = threadIdx.x ? sums[threadIdx.x - 1] : 0u;
    for (unsigned i = b; i < e; i++) {
        const unsigned c = chunkCount[i];
        chunkCount[i] = run;
        run += c;
    }
    if (threadIdx.x == blockDim.x - 1) *nOut = sums[blockDim.x - 1];
}

__global__ void __launch_bounds__(1024) tc_compact_write_kernel(const unsigned *__restrict__ flag, unsigned count,
                                                                const unsigned *__restrict__ chunkStart,
                                                                unsigned *__restrict__ items) {
    const unsigned base = blockIdx.x * kCompactChunk + 4u * threadIdx.x;
    unsigned f[4], local = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        f[k] = (base + k < count && flag[base + k]) ? 1u : 0u;
        local += f[k];
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = local;
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= (unsigned)off) incl += y;
    }
    __shared__ unsigned wsum[32];
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned x = lane < blockDim.x / 32 ? wsum[lane] : 0u;
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= (unsigned)off) x += y;
        }
        wsum[lane] = x;
    }
    __syncthreads();
    unsigned pos = chunkStart[blockIdx.x] + (warp ? wsum[warp - 1] : 0u) + incl - local;
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (f[k]) items[pos++] = base + k;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

static int encode_map(TcState *tc, CUtensorMap *map, const void *base, size_t rows, size_t cols, unsigned boxRows,
                      const char *fn) {
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(cols * sizeof(uint16_t))};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)boxRows};
    cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType dt =
        tc->mode == NOVA_SCORING_FP16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    CUresult res = tc->encode(map, dt, 2, const_cast<void *>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (res != CUDA_SUCCESS) {
        NOVA_ERR(fn, "Failed to encode a TMA tensor map.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    return NOVA_SUCCESS;
}

// (Re)builds A in the element type of the engine's scoring mode.
static int tc_build_operand(BackupEngine &eng, TcState *tc, const char *fn) {
    const DevModel &md = eng.md;
    // A new operand form starts its schedule choice afresh (the margins,
    // and with them the best list length, differ between forms).
    if (tc->mode != eng.scoring) {
        tc->schedFixed = -1;
        tc->tuneNext = 0;
        tc->tuneWarm = false;
    }
    tc->mode = eng.scoring;
    const size_t aElems = (size_t)tc->MZ * tc->rPad * tc->nPad;
    cudaMemsetAsync(tc->A, 0, aElems * sizeof(uint16_t), eng.stream);
    cudaMemsetAsync(tc->a1, 0, (size_t)tc->MZ * tc->rPad * sizeof(float), eng.stream);
    cudaMemsetAsync(tc->a1raw, 0, (size_t)tc->MZ * tc->rPad * sizeof(float), eng.stream);
    cudaMemsetAsync(tc->d1, 0, (size_t)tc->MZ * tc->rPad * sizeof(float), eng.stream);
    cudaMemsetAsync(tc->badModel, 0, sizeof(unsigned), eng.stream);
    // a1 bounds sum_s |A| with A in exact arithmetic: the FP32 sums of
    // non-negative terms are inflated by their worst-case rounding.
    const float slack = 1.0f + (float)(md.n + md.rz * md.ns + 8) * 1.2e-7f;
    // d1 is an FP32 sum of nPad exact non-negative terms.
    const float dslack = 1.0f + (float)(tc->nPad + 8) * 1.2e-7f;
    tc_build_a_kernel<<<md.r * md.m, 256, md.n * sizeof(float), eng.stream>>>(
        md, eng.succLen, eng.suppLen, tc->rPad, tc->nPad, tc->mode == NOVA_SCORING_FP16 ? 1 : 0, tc->A, tc->a1,
        tc->a1raw, tc->d1, slack, dslack, tc->badModel);
    int rc = check_launch(fn, "scoring operand build");
    if (rc != NOVA_SUCCESS) return rc;
    return encode_map(tc, &tc->tmA, tc->A, (size_t)tc->MZ * tc->rPad, tc->nPad, BM, fn);
}

// Dynamic shared memory of every scoring-kernel instantiation (once).
static bool gemm_attributes_set() {
    static std::once_flag once;
    static bool ok = false;
    std::call_once(once, [] {
        const int b = (int)GEMM_SMEM;
        const auto attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
        ok = cudaFuncSetAttribute(tc_score_gemm_kernel<8, SingleUnits>, attr, b) == cudaSuccess &&
             cudaFuncSetAttribute(tc_score_gemm_kernel<16, SingleUnits>, attr, b) == cudaSuccess &&
             cudaFuncSetAttribute(tc_score_gemm_kernel<32, SingleUnits>, attr, b) == cudaSuccess &&
             cudaFuncSetAttribute(tc_score_gemm_kernel<8, BatchUnits>, attr, b) == cudaSuccess &&
             cudaFuncSetAttribute(tc_score_gemm_kernel<16, BatchUnits>, attr, b) == cudaSuccess &&
             cudaFuncSetAttribute(tc_score_gemm_kernel<32, BatchUnits>, attr, b) == cudaSuccess;
        if (!ok) cudaGetLastError();
    });
    return ok;
}

int tc_build(BackupEngine &eng, const char *fn) {
    if (eng.tc) return NOVA_SUCCESS;
    const DevModel &md = eng.md;
    std::unique_ptr<TcState> tc(new TcState());
    tc->nPad = round_up(md.n, BK);
    tc->rPad = round_up(md.r, BM);
    tc->capN = round_up(md.r, BN);
    tc->MZ = md.m * md.z;
    tc->mTiles = (unsigned)(tc->rPad / BM);
    const size_t aElems = (size_t)tc->MZ * tc->rPad * tc->nPad;
    size_t freeB = 0, totalB = 0;
    cudaMemGetInfo(&freeB, &totalB);
    const size_t slots = (size_t)tc->MZ * md.r * MAX_LISTS;
    const size_t need = aElems * 2 + tc->capN * tc->nPad * 4 + slots * (MAX_TOPK * 8 + 4) + (size_t)tc->MZ * md.r * 12;
    if (need + (256ull << 20) > freeB) {
        NOVA_ERR(fn, "Not enough device memory for the tensor-core operands; using exact scoring.");
        return NOVA_ERROR_DEVICE_MALLOC;
    }
    void *fnPtr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fnPtr, 12000, cudaEnableDefault, &q) !=
            cudaSuccess || q != cudaDriverEntryPointSuccess || fnPtr == nullptr) {
        cudaGetLastError();
        NOVA_ERR(fn, "cuTensorMapEncodeTiled is not available.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    tc->encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fnPtr);
    int rc;
    if ((rc = dev_alloc(&tc->A, aElems, fn, "the tensor-core scoring operand")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->a1, (size_t)tc->MZ * tc->rPad, fn, "the row bounds")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->a1raw, (size_t)tc->MZ * tc->rPad, fn, "the row bounds")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->d1, (size_t)tc->MZ * tc->rPad, fn, "the row bounds")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->Gb, tc->capN * tc->nPad * 2, fn, "the packed alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->shift, md.n, fn, "the alpha shift")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->scal, 8, fn, "the scoring scalars")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->candV, slots * MAX_TOPK, fn, "the candidate scores")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->candU, slots * MAX_TOPK, fn, "the candidate alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->candX, slots, fn, "the dropped-score bounds")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->rowFlag, (size_t)tc->MZ * md.r, fn, "the exact-scan flags")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->rowCand, (size_t)tc->MZ * md.r, fn, "the per-row re-score counts")) != NOVA_SUCCESS)
        return rc;
    if ((rc = dev_alloc(&tc->rowList, (size_t)tc->MZ * md.r, fn, "the exact-scan rows")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&tc->chunkCount, ceil_div((size_t)tc->MZ * md.r, kCompactChunk), fn,
                        "the exact-scan chunk counts")) != NOVA_SUCCESS)
        return rc;
    if ((rc = dev_alloc(&tc->badModel, 1, fn, "the model check")) != NOVA_SUCCESS) return rc;
    if ((rc = tc_build_operand(eng, tc.get(), fn)) != NOVA_SUCCESS) return rc;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, 0);
    tc->numSMs = prop.multiProcessorCount;
    cudaEventCreate(&tc->g0);
    cudaEventCreate(&tc->g1);
    if (!gemm_attributes_set()) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to configure the scoring kernel's shared memory.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    eng.tc = tc.release();
    return sync_device(fn);
}

int tc_prepare(BackupEngine &eng, const float *src, unsigned nU, const char *fn) {
    int rc;
    if (!eng.tc && (rc = tc_build(eng, fn)) != NOVA_SUCCESS) return rc;
    TcState *tc = eng.tc;
    if (tc->mode != eng.scoring && (rc = tc_build_operand(eng, tc, fn)) != NOVA_SUCCESS) return rc;
    tc->src = src;
    const DevModel &md = eng.md;
    const bool fp16 = tc->mode == NOVA_SCORING_FP16;
    // BF16 carries the alphas as two BF16 terms (split); FP16 as one.
    const unsigned kSplit = fp16 ? 1u : 2u;
    const size_t nPadRows = round_up(nU, BN);
    const unsigned nTiles = (unsigned)(nPadRows / BN);
    // ---- pack the shifted, scaled unique alphas ----
    cudaMemsetAsync(tc->scal, 0, 8 * sizeof(unsigned), eng.stream);
    tc_shift_kernel<<<md.n, 256, 0, eng.stream>>>(eng.Gt, eng.gtCols, md.n, nU, tc->shift, tc->scal);
    if ((rc = check_launch(fn, "alpha shift")) != NOVA_SUCCESS) return rc;
    tc_gscale_kernel<<<1, 1, 0, eng.stream>>>(tc->scal);
    if ((rc = check_launch(fn, "alpha scale")) != NOVA_SUCCESS) return rc;
    tc_pack_kernel<<<(unsigned)nPadRows, 256, 0, eng.stream>>>(src, md.n, tc->nPad, eng.uniqJ, nU, tc->shift,
                                                              fp16 ? 1 : 0, kSplit == 2u ? 1 : 0, tc->Gb, tc->scal);
    if ((rc = check_launch(fn, "alpha packing")) != NOVA_SUCCESS) return rc;
    // The row bound is a1 * escale + d1 * dscale (packed units), with
    // escale = U * gmax + gN * Gmax * gscale and dscale = gmax (1 + 2^-22).
    // Against the reference's FP32 score, the tensor-core score of a row
    // (shifted by a row constant) differs by at most
    //  * sum_s |A - Ahalf| |alpha - c|  <= d1 gmax: A's operand rounding,
    //    measured per row when A was built;
    //  * epsA a1 gmax: the FP32 build of A itself;
    //  * (1 + uA)(uG + 2^-23) a1 gmax: the alphas' rounding to FP16 (uG =
    //    2^-11, plus the absolute error of FP16 subnormals, below 2^-25 per
    //    entry) or to the hi + lo BF16 pair (uG = 2^-16), and the FP32
    //    rounding of alpha - c;
    //  * the accumulation: each tcgen05.mma step (K=16) adds at most 2^-22 of
    //    the running sum of magnitudes, over kSplit * nPad / 16 steps;
    //  * gN a1 Gmax: the reference's own rounding over ns + rz + 3 operations.
    // uA is A's unit roundoff (2^-11 FP16, 2^-8 BF16).
    const double u24 = 1.0 / 16777216.0;
    const double epsA = (double)(md.rz * md.ns + 4) * u24;
    const double uA = fp16 ? 1.0 / 2048.0 : 1.0 / 256.0;
    const double uG = fp16 ? 1.0 / 2048.0 : 1.0 / 65536.0;
    const double steps = (double)kSplit * (double)tc->nPad / 16.0 + 2.0;
    const float U = (float)(epsA * (1.0 + 2.0 * u24) + (1.0 + uA) * (uG + 2.0 * u24) +
                            steps / 4194304.0 * (1.0 + uA) * (1.0 + uG) * (1.0 + 2.0 * u24) +
                            (fp16 ? (double)tc->nPad / 33554432.0 / 8192.0 : 0.0) + 1.0 / 1048576.0);
    const float gN = (float)((double)(md.ns + md.rz + 3) * u24 * 1.01);
    tc_escale_kernel<<<1, 1, 0, eng.stream>>>(tc->scal, U, gN);
    if ((rc = check_launch(fn, "margin")) != NOVA_SUCCESS) return rc;
    // ---- schedule and the alphas' tensor map ----
    TcState::Launch &L = tc->last;
    if ((rc = encode_map(tc, &L.tmB, tc->Gb, nPadRows, tc->nPad * kSplit, BN, fn)) != NOVA_SUCCESS) return rc;
    // Each alpha group leaves two lists per row (one per epilogue half).
    if (tc->schedFixed < 0 && tc->nPad > kTuneMaxNPad) tc->schedFixed = fp16 ? kDeepScheduleFp16 : kDeepScheduleBf16;
    const TcSchedule sched = kSchedules[tc->schedFixed >= 0 ? tc->schedFixed : (tc->tuneWarm ? (int)tc->tuneNext : 0)];
    L.nU = nU;
    L.nTiles = nTiles;
    L.groups = std::max(1u, std::min<unsigned>(sched.groups, nTiles));
    L.lists = 2u * L.groups;
    L.topk = sched.topk;
    L.kSplit = kSplit;
    L.fp16 = fp16;
    tc->groupsUsed = L.groups;
    return NOVA_SUCCESS;
}

// The scoring GEMM of one prepared solver on its stream.
int tc_gemm(BackupEngine &eng, bool timed, const char *fn) {
    TcState *tc = eng.tc;
    const TcState::Launch &L = tc->last;
    const unsigned totalUnits = tc->MZ * tc->mTiles * L.groups;
    const unsigned grid = std::min<unsigned>(totalUnits, (unsigned)tc->numSMs);
    if (timed) cudaEventRecord(tc->g0, eng.stream);
    auto gemm = L.topk == 32u ? tc_score_gemm_kernel<32, SingleUnits>
                : (L.topk == 16u ? tc_score_gemm_kernel<16, SingleUnits> : tc_score_gemm_kernel<8, SingleUnits>);
    const SingleUnits units{tc->MZ, (unsigned)tc->rPad, eng.md.r, tc->mTiles, L.nTiles, L.groups, L.nU,
                            (unsigned)(tc->nPad / BK), L.kSplit, tc->a1, tc->d1, tc->scal, tc->candV, tc->candU,
                            tc->candX};
    gemm<<<grid, GEMM_THREADS, GEMM_SMEM, eng.stream>>>(tc->tmA, L.tmB, make_idesc(L.fp16 ? 0u : 1u), units);
    int rc = check_launch(fn, "tensor-core scoring");
    if (rc != NOVA_SUCCESS) return rc;
    if (timed) cudaEventRecord(tc->g1, eng.stream);
    return NOVA_SUCCESS;
}

// After the GEMM: merge the lists, apply the margin, re-score near ties
// exactly, and list the rows left to the exact scan (count in eng.itemCount).
int tc_finish(BackupEngine &eng, const char *fn) {
    TcState *tc = eng.tc;
    const TcState::Launch &L = tc->last;
    const DevModel &md = eng.md;
    int rc;
    const size_t rows = (size_t)tc->MZ * md.r;
    cudaMemsetAsync(tc->rowFlag, 0, rows * sizeof(unsigned), eng.stream);
    const DirectScorer ds{eng.succLen, eng.C3, tc->src};
    auto merge = eng.useProjNow ? tc_merge_kernel<false> : tc_merge_kernel<true>;
    const size_t mergeSmem = eng.useProjNow ? 0 : (256 / 32) * 1024 * sizeof(float);
    merge<<<(unsigned)ceil_div(rows * 32, 256), 256, mergeSmem, eng.stream>>>(
        md, eng.suppLen, eng.useProjNow ? eng.proj_view() : ProjView{}, ds, eng.uniqJ, L.lists, L.topk, tc->rPad,
        tc->a1, tc->d1, tc->a1raw, tc->scal, tc->candV, tc->candU, tc->candX, eng.ustar, eng.jstar, tc->rowFlag,
        tc->rowCand, tc->scal + 3, tc->badModel);
    if ((rc = check_launch(fn, "candidate merge")) != NOVA_SUCCESS) return rc;
    // The list can hold every row: it is sized m*z*r like the flags.
    const unsigned nChunks = ceil_div(rows, kCompactChunk);
    tc_compact_count_kernel<<<nChunks, 1024, 0, eng.stream>>>(tc->rowFlag, (unsigned)rows, tc->chunkCount);
    if ((rc = check_launch(fn, "exact-scan list (count)")) != NOVA_SUCCESS) return rc;
    tc_compact_scan_kernel<<<1, 1024, 0, eng.stream>>>(tc->chunkCount, nChunks, eng.itemCount);
    if ((rc = check_launch(fn, "exact-scan list (scan)")) != NOVA_SUCCESS) return rc;
    tc_compact_write_kernel<<<nChunks, 1024, 0, eng.stream>>>(tc->rowFlag, (unsigned)rows, tc->chunkCount,
                                                              tc->rowList);
    return check_launch(fn, "exact-scan list (write)");
}

// Flag the (belief, action) item of every listed row.
__global__ void tc_row_items_kernel(const unsigned *__restrict__ rowList, unsigned nRows, unsigned r, unsigned m,
                                    unsigned z, unsigned *__restrict__ itemFlag) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nRows) return;
    const unsigned row = rowList[t];
    const unsigned ao = row / r, i = row % r;
    itemFlag[(size_t)i * m + ao / z] = 1u;
}

// The distinct (belief, action) items of the listed rows, in increasing
// order, into eng.items (count in eng.itemCount). The row flags are free
// again once the row list is written, and hold the item flags.
int tc_rows_to_items(BackupEngine &eng, const unsigned *rowList, unsigned nRows, const char *fn) {
    TcState *tc = eng.tc;
    const DevModel &md = eng.md;
    const unsigned count = md.r * md.m;
    int rc;
    cudaMemsetAsync(tc->rowFlag, 0, (size_t)count * sizeof(unsigned), eng.stream);
    tc_row_items_kernel<<<ceil_div(nRows, 256), 256, 0, eng.stream>>>(rowList, nRows, md.r, md.m, md.z,
                                                                      tc->rowFlag);
    if ((rc = check_launch(fn, "rows to items")) != NOVA_SUCCESS) return rc;
    const unsigned nChunks = ceil_div(count, kCompactChunk);
    tc_compact_count_kernel<<<nChunks, 1024, 0, eng.stream>>>(tc->rowFlag, count, tc->chunkCount);
    if ((rc = check_launch(fn, "item list (count)")) != NOVA_SUCCESS) return rc;
    tc_compact_scan_kernel<<<1, 1024, 0, eng.stream>>>(tc->chunkCount, nChunks, eng.itemCount);
    if ((rc = check_launch(fn, "item list (scan)")) != NOVA_SUCCESS) return rc;
    tc_compact_write_kernel<<<nChunks, 1024, 0, eng.stream>>>(tc->rowFlag, count, tc->chunkCount, eng.items);
    return check_launch(fn, "item list (write)");
}

int tc_score_launch(BackupEngine &eng, const float *src, unsigned nU, bool timed, const char *fn) {
    int rc;
    if ((rc = tc_prepare(eng, src, nU, fn)) != NOVA_SUCCESS) return rc;
    if ((rc = tc_gemm(eng, timed, fn)) != NOVA_SUCCESS) return rc;
    return tc_finish(eng, fn);
}

// ---------------------------------------------------------------------------
// Batched scoring: one persistent launch over the work units of many solvers
// ---------------------------------------------------------------------------

struct TcBatch {
    struct Group {
        unsigned topk = 0, totalUnits = 0, nModels = 0;
        bool fp16 = true;
        BatchModel *models = nullptr;   // device work table
    };
    std::vector<Group> groups;   // one per list length and operand form
    int numSMs = 0;
    ~TcBatch() {
        for (auto &g : groups) cudaFree(g.models);
    }
};

int tc_batch_create(BackupEngine *const *engs, unsigned count, TcBatch **out, const char *fn) {
    std::unique_ptr<TcBatch> b(new TcBatch());
    std::vector<std::vector<BatchModel>> host;
    for (unsigned k = 0; k < count; k++) {
        const BackupEngine &e = *engs[k];
        const TcState *tc = e.tc;
        if (tc == nullptr || tc->last.topk == 0) {
            NOVA_ERR(fn, "A solver of the batch has no prepared tensor-core launch.");
            return NOVA_ERROR_INVALID_DATA;
        }
        const TcState::Launch &L = tc->last;
        if (L.topk != 8u && L.topk != 16u && L.topk != 32u) {
            NOVA_ERR(fn, "Unsupported candidate-list length for a batched launch.");
            return NOVA_ERROR_INVALID_DATA;
        }
        size_t gi = 0;
        while (gi < b->groups.size() && (b->groups[gi].topk != L.topk || b->groups[gi].fp16 != L.fp16)) gi++;
        if (gi == b->groups.size()) {
            b->groups.emplace_back();
            b->groups.back().topk = L.topk;
            b->groups.back().fp16 = L.fp16;
            host.emplace_back();
        }
        TcBatch::Group &g = b->groups[gi];
        BatchModel m;
        memset(&m, 0, sizeof(m));
        m.tmA = tc->tmA;
        m.tmB = L.tmB;
        m.unitStart = g.totalUnits;
        m.MZ = tc->MZ;
        m.rPad = (unsigned)tc->rPad;
        m.r = e.md.r;
        m.mTiles = tc->mTiles;
        m.nTiles = L.nTiles;
        m.groups = L.groups;
        m.nU = L.nU;
        m.kBlocks = (unsigned)(tc->nPad / BK);
        m.kSplit = L.kSplit;
        m.a1 = tc->a1; m.d1 = tc->d1; m.scal = tc->scal;
        m.candV = tc->candV; m.candU = tc->candU; m.candX = tc->candX;
        const unsigned long long units = (unsigned long long)m.MZ * m.mTiles * m.groups;
        if ((unsigned long long)g.totalUnits + units >= (1ull << 31)) {
            NOVA_ERR(fn, "Too many work units for one batched launch.");
            return NOVA_ERROR_INVALID_DATA;
        }
        g.totalUnits += (unsigned)units;
        g.nModels++;
        host[gi].push_back(m);
        b->numSMs = tc->numSMs;
    }
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        int rc;
        if ((rc = dev_alloc(&b->groups[gi].models, host[gi].size(), fn, "the batch work table")) != NOVA_SUCCESS)
            return rc;
        if ((rc = h2d(b->groups[gi].models, host[gi].data(), host[gi].size() * sizeof(BatchModel), fn,
                      "the batch work table")) != NOVA_SUCCESS)
            return rc;
    }
    *out = b.release();
    return NOVA_SUCCESS;
}

int tc_batch_gemm(TcBatch *b, cudaStream_t stream, const char *fn) {
    for (const auto &g : b->groups) {
        if (g.totalUnits == 0) continue;
        const BatchUnits units{g.models, g.nModels, g.totalUnits};
        const unsigned grid = std::min<unsigned>(g.totalUnits, (unsigned)b->numSMs);
        CUtensorMap unused;
        memset(&unused, 0, sizeof(unused));
        auto kern = g.topk == 32u ? tc_score_gemm_kernel<32, BatchUnits>
                    : (g.topk == 16u ? tc_score_gemm_kernel<16, BatchUnits> : tc_score_gemm_kernel<8, BatchUnits>);
        kern<<<grid, GEMM_THREADS, GEMM_SMEM, stream>>>(unused, unused, make_idesc(g.fp16 ? 0u : 1u), units);
        int rc = check_launch(fn, "batched tensor-core scoring");
        if (rc != NOVA_SUCCESS) return rc;
    }
    return NOVA_SUCCESS;
}

void tc_batch_release(TcBatch *b) { delete b; }

bool tc_schedule_fixed(const BackupEngine &eng) {
    // Fixed, and the operand is built for the solver's current mode (a
    // rebuild must not end up inside a captured update).
    return eng.tc != nullptr && eng.tc->schedFixed >= 0 && eng.tc->mode == eng.scoring;
}

const unsigned *tc_row_list(const BackupEngine &eng) { return eng.tc ? eng.tc->rowList : nullptr; }

int tc_score(BackupEngine &eng, const float *src, unsigned nU, unsigned *nRows, const unsigned **rowList,
             const char *fn) {
    int rc;
    if ((rc = tc_score_launch(eng, src, nU, true, fn)) != NOVA_SUCCESS) return rc;
    TcState *tc = eng.tc;
    unsigned h[8];
    unsigned cnt = 0;
    if (cudaMemcpyAsync(h, tc->scal, sizeof(h), cudaMemcpyDeviceToHost, eng.stream) != cudaSuccess ||
            cudaMemcpyAsync(&cnt, eng.itemCount, sizeof(unsigned), cudaMemcpyDeviceToHost, eng.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(eng.stream) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to read the scoring counters.");
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    if (tc_device_error() != 0) {
        NOVA_ERR(fn, "The tensor-core scoring kernel timed out waiting on a barrier.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    *nRows = cnt;
    *rowList = tc->rowList;
    eng.stats.rowsMultiCand = h[3];
    eng.stats.candidates = h[4];
    cudaEventElapsedTime(&eng.stats.msGemm, tc->g0, tc->g1);
    eng.stats.tcGroups = tc->groupsUsed;
    return NOVA_SUCCESS;
}

int tc_row_detail(const BackupEngine &eng, unsigned *candidates, unsigned *exactRows, const char *fn) {
    const TcState *tc = eng.tc;
    const DevModel &md = eng.md;
    const size_t rows = (size_t)md.m * md.z * md.r;
    std::vector<unsigned> cand(rows), flag(rows);
    if (cudaStreamSynchronize(eng.stream) != cudaSuccess ||
            cudaMemcpy(cand.data(), tc->rowCand, rows * sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(flag.data(), tc->rowFlag, rows * sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to read the per-row scoring detail.");
        return NOVA_ERROR_MEMCPY_TO_HOST;
    }
    for (unsigned i = 0; i < md.r; i++) { candidates[i] = 0; exactRows[i] = 0; }
    for (size_t row = 0; row < rows; row++) {   // row = (a*z + o) * r + i
        const unsigned i = (unsigned)(row % md.r);
        candidates[i] += cand[row];
        exactRows[i] += flag[row] ? 1u : 0u;
    }
    return NOVA_SUCCESS;
}

float tc_tuned_cost(const BackupEngine &eng) {
    const TcState *tc = eng.tc;
    if (tc == nullptr || tc->schedFixed < 0 || tc->schedFixed >= kTunedSchedules ||
            tc->tuneNext < (unsigned)kTunedSchedules)
        return -1.0f;
    return tc->tuneCost[tc->schedFixed];
}

void tc_tune_feedback(BackupEngine &eng, float msScoring, unsigned nU) {
    TcState *tc = eng.tc;
    if (tc == nullptr || tc->schedFixed >= 0 || nU == 0) return;
    if (!tc->tuneWarm) {
        tc->tuneWarm = true;
        return;
    }
    tc->tuneCost[tc->tuneNext] = msScoring / (float)nU;
    if (++tc->tuneNext < (unsigned)kTunedSchedules) return;
    unsigned best = 0;
    for (unsigned k = 1; k < (unsigned)kTunedSchedules; k++)
        if (tc->tuneCost[k] < tc->tuneCost[best]) best = k;
    tc->schedFixed = (int)best;
}

}  // namespace nova_gb300
