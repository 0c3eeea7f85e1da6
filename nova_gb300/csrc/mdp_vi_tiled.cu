// nova-gb300: column-tiled Bellman sweep for large sparse MDPs.
//
// The per-row sweep (mdp_vi.cu) gathers V[S(s,a,l)] straight from L2: at
// n = 2^20, m = 8, ns = 16 that is 134M random 4-byte requests per sweep,
// and L1/L2 request throughput, not HBM, bounds it. This sweep turns the
// gathers into shared-memory reads:
//
//   * Source states are cut into blocks of Sb states (one CTA at a time per
//     block; its m*Sb partial sums Q(s,a) live in shared memory, seeded with
//     R(s,a)). Successor states are cut into tiles of Vt states. One warp of
//     the CTA stages V tile after tile into a ring of shared-memory buffers
//     with bulk copies (cp.async.bulk, completion on an mbarrier); the other
//     31 warps each own a fixed range of the block's rows and add, tile
//     after tile, the products of their rows' successors that fall in the
//     tile. A warp releases a buffer (mbarrier arrive) when it is done with
//     it, so warps run independently of each other, up to the ring's depth.
//   * A row's successors inside one tile form a run (consecutive in the
//     row's list). The plan, built once per solver, stores for every slice
//     (block, tile, warp) the 8-byte records {row << 16 | offset in tile,
//     fl(gamma * T)} (the reference's first rounding, done once) of its
//     runs, level after level: level q holds the q-th record of every run
//     with more than q records, runs ordered by length (longest first), so
//     run j has its level-q record at position j of level q. Lane l of the
//     warp applies runs l, l + 32, ... of the slice, each run's records in
//     list order; the runs of a slice have distinct rows, and a warp's
//     slices run in tile order, so every row receives its products in list
//     order. Records stream from HBM exactly once per sweep (the same 8
//     bytes per entry as S and T): each warp loads its next slice's records
//     while it applies the current one, and the staging warp prefetches the
//     records of the tile after that into L2 with one bulk prefetch.
//   * The single-record runs of a slice are dealt round-robin over the 32
//     shared-memory banks of their partial sums (row mod 32), so a warp's 32
//     runs of one step update distinct banks.
//
// Order of operations: the reference computes Q = R(s,a), then for each
// successor in list order Q += (gamma * T) * V[s'] (mdp_vi_cpu.cpp:45-52).
// When every row's successors are listed in ascending state order, tile
// order is list order, so this sweep performs the same roundings in the same
// order and its results are bit-identical. The plan builder checks that;
// models with unsorted rows keep the per-row sweep.
//
// Every mbarrier wait is bounded (about 2 s); a wait that runs out raises
// the CTA's abort flag and the state's error word, the warps stop, the
// staging warp waits (bounded) for its copies in flight, and the host
// reports NOVA_ERROR_KERNEL_EXECUTION.

#include "vi.h"

#include <algorithm>
#include <atomic>

#include <nova/nova_gb300.h>

using nova::MDP;

namespace nova_gb300 {

namespace {

constexpr unsigned kThreads = 1024;
constexpr unsigned kWarps = kThreads / 32;
constexpr unsigned kRowWarps = kWarps - 1;        // warps that apply records; the last one stages V
constexpr int kSteps = 4;                         // groups of 32 records a warp holds per slice in registers
constexpr unsigned kStages = 3;                   // V tiles in flight
constexpr unsigned kMaxRows = 65535u;             // rows of one block (16-bit row field)
constexpr unsigned kMaxLevels = 31u;              // longest run of one row inside one tile
constexpr unsigned kDefaultTileStates = 8192u;
constexpr unsigned long long kAutoMinEntries = 1ull << 22;
constexpr long long kWaitCycles = 4000000000ll;   // ~2 s at 2 GHz
constexpr size_t kBarrierBytes = 64;              // full[kStages], empty[kStages], abort flag

std::atomic<unsigned> g_mode{NOVA_VI_TILING_AUTO};
std::atomic<unsigned> g_tile_states{0};
std::atomic<unsigned> g_last_status{0};

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

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
// Bounded wait: false (after raising the abort flag and the error word) if
// the phase does not complete in ~2 s, or if the CTA already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abortFlag,
                                          ViDeviceState *st) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abortFlag) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abortFlag = 1;
            atomicExch(&st->err, 1u);
            return false;
        }
    }
}
// Bulk copy global -> shared (16-byte aligned, size a multiple of 16)
// completing on an mbarrier.
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}
// Bulk prefetch of a record range into L2 (the record array has two spare
// records at its end for the rounding up to 16 bytes).
__device__ __forceinline__ void prefetch_l2(const uint2 *rec, unsigned b, unsigned e) {
    if (e <= b) return;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(rec + b) & ~(uintptr_t)15;
    const uintptr_t hi = (reinterpret_cast<uintptr_t>(rec + e) + 15) & ~(uintptr_t)15;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
}

constexpr uint2 kNoRecord = {0xFFFFFFFFu, 0u};

// What a lane holds for one slice: the slice's first record and run counts
// (n0 runs, n1 of them with a second record, n2 with a third), the level-0
// records of its runs lane + 32 i (i < kSteps) and the level-1 record of run
// `lane`.
struct SliceRegs {
    uint2 r[kSteps];
    uint2 r1;
    unsigned start, n0, n1, n2;
};
// hdr = {first record, n0, n1, n2} of the slice.
__device__ __forceinline__ void load_slice(SliceRegs &g, const uint2 *__restrict__ rec, uint4 hdr, unsigned lane) {
    g.start = hdr.x;
    g.n0 = hdr.y;
    g.n1 = hdr.z;
    g.n2 = hdr.w;
#pragma unroll
    for (int i = 0; i < kSteps; i++) {
        const unsigned j = lane + 32u * i;
        g.r[i] = j < g.n0 ? __ldg(rec + g.start + j) : kNoRecord;
    }
    g.r1 = lane < g.n1 ? __ldg(rec + g.start + g.n0 + lane) : kNoRecord;
}

// part[row] += fl(gamma*T) * V[s'] for one record.
__device__ __forceinline__ void apply_record(uint2 r, const float *vtile, unsigned tileLen, float *part,
                                             unsigned rows) {
    const unsigned row = r.x >> 16, off = r.x & 0xFFFFu;
    if (row < rows && off < tileLen) part[row] = fadd(part[row], fmul(__uint_as_float(r.y), vtile[off]));
}

// Records of run j from level 1 on (run j has at least two), in list order.
// Only the rare runs of three or more records read further level counts.
__device__ __forceinline__ void apply_long_run(const SliceRegs &g, unsigned j, uint2 first1,
                                               const uint2 *__restrict__ rec, const unsigned *__restrict__ levelCnt,
                                               unsigned L, unsigned slice, const float *vtile, unsigned tileLen,
                                               float *part, unsigned rows) {
    apply_record(first1, vtile, tileLen, part, rows);
    if (j >= g.n2) return;
    unsigned base = g.n0 + g.n1;
    apply_record(__ldg(rec + g.start + base + j), vtile, tileLen, part, rows);
    base += g.n2;
    for (unsigned lv = 3; lv < L; lv++) {
        const unsigned nq = __ldg(levelCnt + (size_t)slice * L + lv);
        if (j >= nq) break;
        apply_record(__ldg(rec + g.start + base + j), vtile, tileLen, part, rows);
        base += nq;
    }
}

// One slice: the level-0 record of every run, then the further records of
// the long runs (runs 0 .. n1-1), each in list order after its level-0
// record (the same lane applies both; no other run of the slice has that
// row).
__device__ __forceinline__ void apply_slice(const SliceRegs &g, const uint2 *__restrict__ rec,
                                            const unsigned *__restrict__ levelCnt, unsigned L, unsigned slice,
                                            const float *vtile, unsigned tileLen, float *part, unsigned rows,
                                            unsigned lane) {
#pragma unroll
    for (int i = 0; i < kSteps; i++)
        if (lane + 32u * i < g.n0) apply_record(g.r[i], vtile, tileLen, part, rows);
    for (unsigned j = lane + 32u * kSteps; j < g.n0; j += 32u)
        apply_record(__ldg(rec + g.start + j), vtile, tileLen, part, rows);
    if (lane < g.n1) apply_long_run(g, lane, g.r1, rec, levelCnt, L, slice, vtile, tileLen, part, rows);
    for (unsigned j = lane + 32u; j < g.n1; j += 32u)
        apply_long_run(g, j, __ldg(rec + g.start + g.n0 + j), rec, levelCnt, L, slice, vtile, tileLen, part, rows);
}

// One tile of a row warp: load the next slice (and the header after it),
// wait for the V tile, apply the current slice, release the buffer.
__device__ __forceinline__ bool row_warp_tile(unsigned t, unsigned T, const SliceRegs &cur, SliceRegs &nxt,
                                              uint4 &hNext, unsigned sl0, const uint2 *__restrict__ rec,
                                              const uint4 *__restrict__ sliceHdr,
                                              const unsigned *__restrict__ levelCnt, unsigned L, const float *vt,
                                              unsigned Vt, unsigned n, float *part, unsigned rows, uint64_t *bars,
                                              unsigned &sg, unsigned &ph, volatile int *abortFlag,
                                              ViDeviceState *st, unsigned lane) {
    if (t + 1 < T) {
        load_slice(nxt, rec, hNext, lane);
        hNext = t + 2 < T ? __ldg(sliceHdr + sl0 + (t + 2) * kRowWarps) : make_uint4(0u, 0u, 0u, 0u);
    }
    if (!mbar_wait(smem_addr(&bars[sg]), ph, abortFlag, st)) return false;
    apply_slice(cur, rec, levelCnt, L, sl0 + t * kRowWarps, vt + (size_t)sg * Vt, min(Vt, n - t * Vt), part, rows,
                lane);
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_addr(&bars[kStages + sg]));
    if (++sg == kStages) { sg = 0; ph ^= 1u; }
    return true;
}

__global__ void __launch_bounds__(kThreads, 1) bellman_tiled_kernel(
        unsigned n, unsigned m, unsigned Vt, unsigned T, unsigned Sb, unsigned blocks, unsigned L,
        const uint2 *__restrict__ rec, const unsigned *__restrict__ sliceStart, const uint4 *__restrict__ sliceHdr,
        const unsigned *__restrict__ levelCnt, const float *__restrict__ R, const float *__restrict__ V,
        float *__restrict__ Vp, unsigned *__restrict__ pi, ViDeviceState *st, double tol, int early_exit) {
    if (early_exit && *(volatile unsigned *)&st->converged) return;  // uniform across the grid
    extern __shared__ __align__(128) unsigned char smem[];
    float *vt = reinterpret_cast<float *>(smem);                              // [kStages][Vt]
    float *part = vt + (size_t)kStages * Vt;                                  // [Sb*m]
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + (((size_t)kStages * Vt + (size_t)Sb * m) * 4 + 15) /
                                                             16 * 16);
    volatile int *abortFlag = reinterpret_cast<volatile int *>(bars + 2 * kStages);
    const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (unsigned s = 0; s < kStages; s++) {
            mbar_init(smem_addr(&bars[s]), 1);                 // full: the staging lane's arrival + bytes
            mbar_init(smem_addr(&bars[kStages + s]), kRowWarps);  // empty: one arrival per row warp
        }
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned stage = 0, phase = 0;   // ring position, advanced identically by every warp
    unsigned lastPar[kStages];       // staging lane: parity of the last copy issued per stage (2: none)
#pragma unroll
    for (unsigned s = 0; s < kStages; s++) lastPar[s] = 2u;
    double local = 0.0;
    for (unsigned blk = blockIdx.x; blk < blocks && !*abortFlag; blk += gridDim.x) {
        const unsigned s0 = blk * Sb;
        const unsigned nsb = min(Sb, n - s0);
        const unsigned rows = nsb * m;
        for (unsigned i = tid; i < rows; i += blockDim.x) part[i] = __ldg(R + (size_t)s0 * m + i);
        __syncthreads();
        const size_t c0 = (size_t)blk * T;
        if (warp == kRowWarps) {
            // ---- staging warp: V tiles into the ring, records into L2 ----
            if (lane == 0) {
                prefetch_l2(rec, __ldg(sliceStart + c0 * kRowWarps), __ldg(sliceStart + (c0 + min(T, 2u)) * kRowWarps));
                unsigned sg = stage, ph = phase;
                for (unsigned t = 0; t < T; t++) {
                    if (!mbar_wait(smem_addr(&bars[kStages + sg]), ph ^ 1u, abortFlag, st)) break;
                    const unsigned base = t * Vt, cnt = min(Vt, n - base);
                    const unsigned body = cnt & ~3u;
                    float *dst = vt + (size_t)sg * Vt;
                    for (unsigned k = body; k < cnt; k++) dst[k] = __ldg(V + base + k);  // tail of the last tile
                    const uint32_t fb = smem_addr(&bars[sg]);
                    mbar_expect_tx(fb, body * 4u);
                    if (body) bulk_copy(smem_addr(dst), V + base, body * 4u, fb);
                    lastPar[sg] = ph;
                    if (t + 2 < T)
                        prefetch_l2(rec, __ldg(sliceStart + (c0 + t + 2) * kRowWarps),
                                    __ldg(sliceStart + (c0 + t + 3) * kRowWarps));
                    if (++sg == kStages) { sg = 0; ph ^= 1u; }
                }
            }
        } else {
            // ---- row warps ----
            // Slice (blk, t) of this warp is sl0 + t * kRowWarps. Records of
            // slice t+1 are loaded while slice t is applied; the two register
            // sets alternate roles, so nothing is copied between tiles.
            const unsigned sl0 = (unsigned)(c0 * kRowWarps) + warp;
            SliceRegs ga, gb;
            load_slice(ga, rec, __ldg(sliceHdr + sl0), lane);
            uint4 hNext = T > 1 ? __ldg(sliceHdr + sl0 + kRowWarps) : make_uint4(0u, 0u, 0u, 0u);
            unsigned sg = stage, ph = phase;
            for (unsigned t = 0; t < T; t += 2) {
                if (!row_warp_tile(t, T, ga, gb, hNext, sl0, rec, sliceHdr, levelCnt, L, vt, Vt, n, part, rows, bars,
                                   sg, ph, abortFlag, st, lane))
                    break;
                if (t + 1 < T && !row_warp_tile(t + 1, T, gb, ga, hNext, sl0, rec, sliceHdr, levelCnt, L, vt, Vt, n,
                                                part, rows, bars, sg, ph, abortFlag, st, lane))
                    break;
            }
        }
        // Every warp advances the ring by the block's T tiles.
        {
            const unsigned adv = stage + T;
            phase ^= (adv / kStages) & 1u;
            stage = adv % kStages;
        }
        __syncthreads();
        if (*abortFlag) break;
        // Action scan of mdp_vi_cpu.cpp:55-58 (lowest action on ties).
        for (unsigned i = tid; i < nsb; i += blockDim.x) {
            const float *qv = part + (size_t)i * m;
            float best = qv[0];
            unsigned besta = 0;
            for (unsigned a = 1; a < m; a++)
                if (qv[a] > best) { best = qv[a]; besta = a; }
            const unsigned s = s0 + i;
            Vp[s] = best;
            pi[s] = besta;
            local = fmax(local, fabs((double)best - (double)__ldg(V + s)));
        }
        __syncthreads();
    }
    if (*abortFlag && warp == kRowWarps && lane == 0) {
        // Let the copies in flight land before the CTA exits (bounded): the
        // last issue on each stage completes the phase of parity lastPar.
        for (unsigned s = 0; s < kStages; s++) {
            if (lastPar[s] > 1u) continue;
            const long long t0 = clock64();
            while (!mbar_try_wait(smem_addr(&bars[s]), lastPar[s]) && clock64() - t0 < kWaitCycles) {
            }
        }
    }
    __syncthreads();
    residual_commit(local, st, gridDim.x, tol, early_exit != 0);
}

// ---------------------------------------------------------------------------
// Plan construction
// ---------------------------------------------------------------------------

// flags[0] = some row is not ascending, flags[1] = a successor index is >= n,
// flags[2] = longest run (successors of one row inside one tile).
__global__ void vi_plan_scan_rows_kernel(unsigned n, unsigned m, unsigned ns, const int *__restrict__ S,
                                         unsigned Vt, unsigned *flags) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)n * m) return;
    const int *Sr = S + row * ns;
    int prev = -1;
    unsigned runTile = 0xFFFFFFFFu, runLen = 0, longest = 0;
    for (unsigned l = 0; l < ns; l++) {
        const int sp = Sr[l];
        if (sp < 0) break;
        if ((unsigned)sp >= n) {
            atomicOr(flags + 1, 1u);
            return;
        }
        if (sp < prev) atomicOr(flags, 1u);
        prev = sp;
        const unsigned t = (unsigned)sp / Vt;
        runLen = t == runTile ? runLen + 1 : 1;
        runTile = t;
        longest = max(longest, runLen);
    }
    if (longest) atomicMax(flags + 2, longest);
}

struct PlanGeometry {
    unsigned n, m, ns, Vt, T, Sb, L, rowsPerWarp;
    float gamma;
    // Slice (block, tile, row warp) of a row of the block.
    __device__ __forceinline__ size_t slice(unsigned blk, unsigned t, unsigned rowLocal) const {
        return ((size_t)blk * T + t) * kRowWarps + rowLocal / rowsPerWarp;
    }
};

// Calls f(tile, first list index, run length) for every run of the row.
template <typename F>
__device__ __forceinline__ void for_each_run(const int *Sr, unsigned ns, unsigned Vt, F f) {
    unsigned l = 0;
    while (l < ns) {
        const int sp = Sr[l];
        if (sp < 0) break;
        const unsigned t = (unsigned)sp / Vt;
        unsigned e = l + 1;
        while (e < ns && Sr[e] >= 0 && (unsigned)Sr[e] / Vt == t) e++;
        f(t, l, e - l);
        l = e;
    }
}

// Per slice: levelCnt[sl*L + q] = runs with more than q records;
// bucket[sl*32 + b] = single-record runs whose partial sum lies in shared-
// memory bank b (row mod 32); longCnt[sl*(L+1) + len] = runs of len >= 2.
__global__ void vi_plan_count_kernel(PlanGeometry g, const int *__restrict__ S, unsigned *__restrict__ levelCnt,
                                     unsigned *__restrict__ bucket, unsigned *__restrict__ longCnt) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)g.n * g.m) return;
    const unsigned blk = (unsigned)(row / g.m) / g.Sb;
    const unsigned rowLocal = (unsigned)(row - (unsigned long long)blk * g.Sb * g.m);
    const int *Sr = S + row * g.ns;
    for_each_run(Sr, g.ns, g.Vt, [&](unsigned t, unsigned, unsigned len) {
        const size_t sl = g.slice(blk, t, rowLocal);
        for (unsigned q = 0; q < len; q++) atomicAdd(levelCnt + sl * g.L + q, 1u);
        if (len == 1) atomicAdd(bucket + sl * 32 + (rowLocal & 31u), 1u);
        else atomicAdd(longCnt + sl * (g.L + 1) + len, 1u);
    });
}

// Per slice: its record count, and the long runs' exclusive prefix by
// length, longest first (in place in longCnt).
__global__ void vi_plan_slice_kernel(size_t nSlices, unsigned L, const unsigned *__restrict__ levelCnt,
                                     unsigned *__restrict__ longCnt, unsigned *__restrict__ sliceSize) {
    const size_t sl = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nSlices) return;
    unsigned total = 0;
    for (unsigned q = 0; q < L; q++) total += levelCnt[sl * L + q];
    sliceSize[sl] = total;
    unsigned run = 0;
    for (unsigned len = L; len >= 2; len--) {
        unsigned *p = longCnt + sl * (L + 1) + len;
        const unsigned v = *p;
        *p = run;
        run += v;
    }
}

// Slice headers for the sweep: {first record, runs, runs with a second
// record, runs with a third record}.
__global__ void vi_plan_hdr_kernel(size_t nSlices, unsigned L, const unsigned *__restrict__ sliceStart,
                                   const unsigned *__restrict__ levelCnt, uint4 *__restrict__ hdr) {
    const size_t sl = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nSlices) return;
    hdr[sl] = make_uint4(sliceStart[sl], levelCnt[sl * L], L > 1 ? levelCnt[sl * L + 1] : 0u,
                         L > 2 ? levelCnt[sl * L + 2] : 0u);
}

// Write every record at its place. The position j of a run in its slice's
// levels: long runs first, by length (ties in the order threads arrive,
// which changes nothing: the rows of one slice are distinct), then the
// single-record runs dealt round-robin over the 32 banks, the k-th run of
// bank b's bucket in round k.
__global__ void vi_plan_fill_kernel(PlanGeometry g, const int *__restrict__ S, const float *__restrict__ Tm,
                                    const unsigned *__restrict__ sliceStart, const unsigned *__restrict__ levelCnt,
                                    const unsigned *__restrict__ bucket, unsigned *__restrict__ ticket,
                                    unsigned *__restrict__ longCnt, uint2 *__restrict__ rec) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)g.n * g.m) return;
    const unsigned blk = (unsigned)(row / g.m) / g.Sb;
    const unsigned rowLocal = (unsigned)(row - (unsigned long long)blk * g.Sb * g.m);
    const int *Sr = S + row * g.ns;
    const float *Tr = Tm + row * g.ns;
    for_each_run(Sr, g.ns, g.Vt, [&](unsigned t, unsigned l0, unsigned len) {
        const size_t sl = g.slice(blk, t, rowLocal);
        unsigned j;
        if (len >= 2) {
            j = atomicAdd(longCnt + sl * (g.L + 1) + len, 1u);
        } else {
            const unsigned qb = rowLocal & 31u;
            const unsigned rank = atomicAdd(ticket + sl * 32 + qb, 1u);
            j = g.L > 1 ? levelCnt[sl * g.L + 1] : 0u;   // the long runs come first
            const unsigned *bs = bucket + sl * 32;
            for (unsigned b = 0; b < 32; b++) {
                const unsigned sz = bs[b];
                j += min(sz, rank) + ((b < qb && sz > rank) ? 1u : 0u);
            }
        }
        unsigned base = sliceStart[sl];
        for (unsigned q = 0; q < len; q++) {
            const unsigned sp = (unsigned)Sr[l0 + q];
            rec[base + j] = make_uint2((rowLocal << 16) | (sp - t * g.Vt), __float_as_uint(fmul(g.gamma, Tr[l0 + q])));
            base += levelCnt[sl * g.L + q];
        }
    });
}

// Exclusive scan of in[0..N) into out[0..N] (out[N] = total) in three
// launches: block sums, a one-block scan of those, then each block's scan.
constexpr unsigned kScanChunk = 4096;  // elements per block (4 per thread)

__global__ void vi_scan_sums_kernel(const unsigned *__restrict__ in, unsigned long long N, unsigned *sums) {
    const unsigned long long base = (unsigned long long)blockIdx.x * kScanChunk;
    unsigned s = 0;
    for (unsigned i = threadIdx.x; i < kScanChunk; i += blockDim.x)
        if (base + i < N) s += in[base + i];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    __shared__ unsigned ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (unsigned w = 0; w < blockDim.x / 32; w++) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

__global__ void vi_scan_small_kernel(const unsigned *__restrict__ counts, unsigned N, unsigned *start) {
    __shared__ unsigned sums[1024];
    const unsigned per = (N + blockDim.x - 1) / blockDim.x;
    const unsigned b = threadIdx.x * per;
    const unsigned e = min(N, b + per);
    unsigned s = 0;
    for (unsigned i = b; i < e; i++) s += counts[i];
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
        start[i] = run;
        run += counts[i];
    }
    if (threadIdx.x == blockDim.x - 1) start[N] = sums[blockDim.x - 1];
}

__global__ void vi_scan_apply_kernel(const unsigned *__restrict__ in, unsigned long long N,
                                     const unsigned *__restrict__ blockStart, unsigned *out) {
    const unsigned long long base = (unsigned long long)blockIdx.x * kScanChunk + 4ull * threadIdx.x;
    unsigned v[4], local = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        v[k] = base + k < N ? in[base + k] : 0u;
        local += v[k];
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
        wsum[lane] = x;  // inclusive over warps
    }
    __syncthreads();
    unsigned run = blockStart[blockIdx.x] + (warp ? wsum[warp - 1] : 0u) + incl - local;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (base + k < N) out[base + k] = run;
        run += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[N] = blockStart[gridDim.x];
}

template <typename T>
bool try_alloc(T **p, size_t count) {
    if (cudaMalloc(reinterpret_cast<void **>(p), std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return false;
    }
    return true;
}

void release(ViTilePlan *plan) {
    cudaFree(plan->rec);
    cudaFree(plan->sliceStart);
    cudaFree(plan->sliceHdr);
    cudaFree(plan->levelCnt);
    cudaFree(plan->flags);
    plan->rec = nullptr;
    plan->sliceStart = plan->levelCnt = plan->flags = nullptr;
    plan->sliceHdr = nullptr;
}

int scan_counts(const unsigned *counts, unsigned long long N, unsigned *out, cudaStream_t stream, const char *fn) {
    const unsigned nb = ceil_div(N, kScanChunk);
    unsigned *sums = nullptr, *sumStart = nullptr;
    if (!try_alloc(&sums, nb) || !try_alloc(&sumStart, (size_t)nb + 1)) {
        cudaFree(sums);
        return NOVA_ERROR_DEVICE_MALLOC;
    }
    int rc;
    vi_scan_sums_kernel<<<nb, 1024, 0, stream>>>(counts, N, sums);
    if ((rc = check_launch(fn, "sweep plan (scan sums)")) == NOVA_SUCCESS) {
        vi_scan_small_kernel<<<1, 1024, 0, stream>>>(sums, nb, sumStart);
        if ((rc = check_launch(fn, "sweep plan (scan)")) == NOVA_SUCCESS) {
            vi_scan_apply_kernel<<<nb, 1024, 0, stream>>>(counts, N, sumStart, out);
            rc = check_launch(fn, "sweep plan (scan apply)");
        }
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    cudaFree(sums);
    cudaFree(sumStart);
    return rc;
}

}  // namespace

ViTilePlan::~ViTilePlan() { release(this); }

int vi_plan_build(ViTilePlan *plan, const MDP *mdp, const int *S, const float *T, cudaStream_t stream,
                  const char *fn) {
    if (plan->status != ViTilePlan::kNotBuilt) return NOVA_SUCCESS;
    plan->status = ViTilePlan::kGather;
    g_last_status.store(ViTilePlan::kGather);
    const unsigned mode = g_mode.load();
    const unsigned n = mdp->n, m = mdp->m, ns = mdp->ns;
    const unsigned long long entries = (unsigned long long)n * m * ns;
    if (mode == NOVA_VI_TILING_NEVER || n == 0 || m == 0 || ns == 0 || S == nullptr || T == nullptr)
        return NOVA_SUCCESS;
    if (mode == NOVA_VI_TILING_AUTO && entries < kAutoMinEntries) return NOVA_SUCCESS;
    if (entries >= 0xFFF00000ull) return NOVA_SUCCESS;  // record positions are 32-bit

    int dev = 0, sms = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return NOVA_SUCCESS;
    }
    const unsigned setting = g_tile_states.load();
    unsigned Vt = setting ? setting : kDefaultTileStates;
    Vt = std::min<unsigned>(Vt, (unsigned)round_up(n, 4));
    const unsigned tiles = ceil_div(n, Vt);
    const size_t fixed = (size_t)kStages * Vt * 4 + 16 + kBarrierBytes;
    const size_t reserve = 1024;  // static shared memory of the residual reduction, with room to spare
    if ((size_t)optin < fixed + reserve + (size_t)m * 4) return NOVA_SUCCESS;
    const unsigned rowsMax = (unsigned)std::min<size_t>(((size_t)optin - fixed - reserve) / 4, kMaxRows);
    const unsigned SbMax = rowsMax / m;
    if (SbMax == 0) return NOVA_SUCCESS;
    const unsigned waves = ceil_div(n, (unsigned long long)sms * SbMax);
    const unsigned Sb = ceil_div(n, (unsigned long long)sms * waves);
    const unsigned blocks = ceil_div(n, Sb);
    const size_t smemBytes = round_up((size_t)kStages * Vt * 4 + (size_t)Sb * m * 4, 16) + kBarrierBytes;

    if (cudaFuncSetAttribute(bellman_tiled_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes) !=
            cudaSuccess) {
        cudaGetLastError();
        return NOVA_SUCCESS;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bellman_tiled_kernel, kThreads, smemBytes) !=
            cudaSuccess || occ < 1) {
        cudaGetLastError();
        return NOVA_SUCCESS;
    }

    // Pass 1: ascending rows, successors in range, longest run.
    if (!try_alloc(&plan->flags, 3)) return NOVA_SUCCESS;
    int rc;
    if (cudaMemsetAsync(plan->flags, 0, 3 * sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan flags.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    const unsigned long long rowsAll = (unsigned long long)n * m;
    const unsigned rowBlocks = ceil_div(rowsAll, 256);
    vi_plan_scan_rows_kernel<<<rowBlocks, 256, 0, stream>>>(n, m, ns, S, Vt, plan->flags);
    if ((rc = check_launch(fn, "sweep plan (rows)")) != NOVA_SUCCESS) { release(plan); return rc; }
    unsigned hflags[3] = {0, 0, 0};
    if ((rc = d2h(hflags, plan->flags, sizeof(hflags), fn, "the sweep plan flags")) != NOVA_SUCCESS) {
        release(plan);
        return rc;
    }
    const unsigned L = std::max(hflags[2], 1u);
    if (hflags[0] != 0 || hflags[1] != 0 || L > kMaxLevels) {
        release(plan);
        return NOVA_SUCCESS;
    }
    const unsigned rowsPerWarp = ceil_div((unsigned long long)Sb * m, kRowWarps);
    const PlanGeometry g{n, m, ns, Vt, tiles, Sb, L, rowsPerWarp, mdp->gamma};
    const unsigned long long nSlices = (unsigned long long)blocks * tiles * kRowWarps;
    if (nSlices * 32ull >= (1ull << 32) || nSlices * (L + 1) >= (1ull << 32)) { release(plan); return NOVA_SUCCESS; }

    // Pass 2: per-slice counts (levels, banks, long runs) and the slice starts.
    unsigned *bucket = nullptr, *ticket = nullptr, *longCnt = nullptr, *sliceSize = nullptr;
    auto freeScratch = [&]() {
        cudaFree(bucket); cudaFree(ticket); cudaFree(longCnt); cudaFree(sliceSize);
        bucket = ticket = longCnt = sliceSize = nullptr;
    };
    if (!try_alloc(&plan->levelCnt, nSlices * L) || !try_alloc(&bucket, nSlices * 32) ||
            !try_alloc(&ticket, nSlices * 32) || !try_alloc(&longCnt, nSlices * (L + 1)) ||
            !try_alloc(&sliceSize, nSlices) || !try_alloc(&plan->sliceStart, nSlices + 1)) {
        freeScratch();
        release(plan);
        return NOVA_SUCCESS;
    }
    if (cudaMemsetAsync(plan->levelCnt, 0, nSlices * L * sizeof(unsigned), stream) != cudaSuccess ||
            cudaMemsetAsync(bucket, 0, nSlices * 32 * sizeof(unsigned), stream) != cudaSuccess ||
            cudaMemsetAsync(ticket, 0, nSlices * 32 * sizeof(unsigned), stream) != cudaSuccess ||
            cudaMemsetAsync(longCnt, 0, nSlices * (L + 1) * sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        freeScratch();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan counters.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    vi_plan_count_kernel<<<rowBlocks, 256, 0, stream>>>(g, S, plan->levelCnt, bucket, longCnt);
    rc = check_launch(fn, "sweep plan (count)");
    if (rc == NOVA_SUCCESS) {
        vi_plan_slice_kernel<<<ceil_div(nSlices, 256), 256, 0, stream>>>((size_t)nSlices, L, plan->levelCnt, longCnt,
                                                                         sliceSize);
        rc = check_launch(fn, "sweep plan (slices)");
    }
    if (rc == NOVA_SUCCESS) rc = scan_counts(sliceSize, nSlices, plan->sliceStart, stream, fn);
    if (rc == NOVA_SUCCESS && !try_alloc(&plan->sliceHdr, nSlices)) rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS) {
        vi_plan_hdr_kernel<<<ceil_div(nSlices, 256), 256, 0, stream>>>((size_t)nSlices, L, plan->sliceStart,
                                                                       plan->levelCnt, plan->sliceHdr);
        rc = check_launch(fn, "sweep plan (headers)");
    }
    unsigned total = 0;
    if (rc == NOVA_SUCCESS)
        rc = d2h(&total, plan->sliceStart + nSlices, sizeof(unsigned), fn, "the sweep plan size");
    // Pass 3: the records (two spare ones at the end for the bulk prefetch).
    if (rc == NOVA_SUCCESS && !try_alloc(&plan->rec, (size_t)total + 2)) rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS &&
            cudaMemsetAsync(plan->rec, 0xFF, ((size_t)total + 2) * sizeof(uint2), stream) != cudaSuccess) {
        cudaGetLastError();
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (rc == NOVA_SUCCESS) {
        vi_plan_fill_kernel<<<rowBlocks, 256, 0, stream>>>(g, S, T, plan->sliceStart, plan->levelCnt, bucket, ticket,
                                                           longCnt, plan->rec);
        rc = check_launch(fn, "sweep plan (fill)");
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    freeScratch();
    if (rc != NOVA_SUCCESS) {
        release(plan);
        return rc == NOVA_ERROR_DEVICE_MALLOC ? NOVA_SUCCESS : rc;  // kGather
    }
    cudaFree(plan->flags);
    plan->flags = nullptr;
    plan->tileStates = Vt;
    plan->tiles = tiles;
    plan->blockStates = Sb;
    plan->blocks = blocks;
    plan->levels = L;
    plan->grid = std::min<unsigned>(blocks, (unsigned)sms * (unsigned)occ);
    plan->smemBytes = smemBytes;
    plan->status = ViTilePlan::kTiled;
    g_last_status.store(ViTilePlan::kTiled);
    return NOVA_SUCCESS;
}

int vi_tiled_sweep(const ViTilePlan *plan, const MDP *mdp, const float *R, const float *V, float *Vp, unsigned *pi,
                   ViDeviceState *st, double tol, int early_exit, cudaStream_t stream, const char *fn) {
    bellman_tiled_kernel<<<plan->grid, kThreads, plan->smemBytes, stream>>>(
        mdp->n, mdp->m, plan->tileStates, plan->tiles, plan->blockStates, plan->blocks, plan->levels, plan->rec,
        plan->sliceStart, plan->sliceHdr, plan->levelCnt, R, V, Vp, pi, st, tol, early_exit);
    return check_launch(fn, "Bellman update (tiled)");
}

unsigned vi_last_plan_status() { return g_last_status.load(); }

int vi_state_error(ViDeviceState *st, const char *fn) {
    unsigned err = 0;
    int rc = d2h(&err, &st->err, sizeof(unsigned), fn, "the sweep error word");
    if (rc != NOVA_SUCCESS) return rc;
    if (err == 0) return NOVA_SUCCESS;
    const unsigned zero = 0;
    h2d(&st->err, &zero, sizeof(unsigned), fn, "the sweep error word");
    NOVA_ERR(fn, "A device-side wait of the Bellman sweep timed out; results are invalid.");
    return NOVA_ERROR_KERNEL_EXECUTION;
}

}  // namespace nova_gb300

extern "C" int mdp_vi_set_tiling_gpu(unsigned int mode, unsigned int tileStates) {
    if (mode > NOVA_VI_TILING_NEVER ||
            (tileStates != 0 && (tileStates % 4 != 0 || tileStates < 64 || tileStates > 16384))) {
        NOVA_ERR("mdp_vi_set_tiling_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    nova_gb300::g_mode.store(mode);
    nova_gb300::g_tile_states.store(tileStates);
    return NOVA_SUCCESS;
}
