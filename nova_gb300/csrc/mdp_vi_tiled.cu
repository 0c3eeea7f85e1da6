// nova-gb300: column-tiled Bellman sweep for large sparse MDPs.
//
// The per-row sweep (mdp_vi.cu) gathers V[S(s,a,l)] straight from L2: at
// n = 2^20, m = 8, ns = 16 that is 134M random 4-byte requests per sweep,
// and L1/L2 request throughput, not HBM, bounds it. This sweep turns the
// gathers into shared-memory reads:
//
//   * Source states are cut into blocks of Sb states (one CTA at a time per
//     block; its m*Sb partial sums Q(s,a) live in shared memory, seeded with
//     R(s,a) by one bulk copy, the next block's R prefetched into L2).
//     Successor states are cut into tiles of Vt states. One warp of the CTA
//     stages V tile after tile into a ring of shared-memory buffers with bulk
//     copies (cp.async.bulk, completion on an mbarrier), across block
//     boundaries; the other kRowWarps warps each own a fixed range of the
//     block's rows and add, tile after tile, the products of their rows'
//     successors that fall in the tile. A warp releases a buffer (mbarrier
//     arrive) when it is done with it, so warps run independently of each
//     other, up to the ring's depth. At the end of a block the row warps
//     meet at a named barrier, scan the actions (Vp, pi, residual) and
//     release Q to the staging warp (mbarrier) for the next block's R.
//   * A row's successors inside one tile form a run (consecutive in the
//     row's list). The plan, built once per solver, stores for every slice
//     (block, tile, warp) the 8-byte records {row << 16 | byte offset in
//     tile, fl(gamma * T)} (the reference's first rounding, done once) of its
//     runs, level after level: level q holds the q-th record of every run
//     with more than q records, runs ordered by length (longest first), so
//     run j has its level-q record at position j of level q. Lane l of the
//     warp applies runs l, l + 32, ... of the slice, each run's records in
//     list order; the runs of a slice have distinct rows, and a warp's
//     slices run in tile order, so every row receives its products in list
//     order. Records stream from HBM exactly once per sweep (the same 8
//     bytes per entry as S and T): each warp loads its next slice's records
//     into registers while it applies the current one, and the staging warp
//     prefetches the records of the tile kAhead tiles on into L2 with one
//     bulk prefetch.
//   * The single-record runs of a slice are dealt round-robin over the 32
//     shared-memory banks of their partial sums (row mod 32), so the 32 runs
//     of one step mostly update distinct banks (a step may span the end of
//     one round and the start of the next).
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

constexpr unsigned kThreads = 512;
constexpr unsigned kWarps = kThreads / 32;
constexpr unsigned kRowWarps = kWarps - 1;        // warps that apply records; the last one stages V
constexpr int kSteps = 9;                         // groups of 32 records a warp holds per slice in registers
constexpr unsigned kStages = 3;                   // V tiles in flight
constexpr unsigned kAhead = 2;                    // tiles between a slice's L2 prefetch and its use
constexpr unsigned kDepth = 1;                    // tiles between a slice's register load and its use
constexpr unsigned kMaxRows = 65535u;             // rows of one block (16-bit row field)
constexpr unsigned kMaxLevels = 31u;              // longest run of one row inside one tile
constexpr unsigned kDefaultTileStates = 8192u;       // default tile: the largest of
constexpr unsigned kMaxDefaultTileStates = 10240u;   // [8192, 10240] with the fewest waves
constexpr unsigned long long kAutoMinEntries = 1ull << 22;
constexpr long long kWaitCycles = 4000000000ll;   // ~2 s at 2 GHz
constexpr size_t kBarrierBytes = 96;              // full[kStages], empty[kStages], qReady, qFree, two flags

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
// try_wait, with a suspend-time hint when kHintNs > 0: a waiting thread may
// sleep up to the hint until the phase completes instead of spinning on
// issue slots.
constexpr uint32_t kSuspendNs = 20000;
template <uint32_t kHintNs>
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    if constexpr (kHintNs > 0) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity), "r"(kHintNs)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
    }
    return ok != 0;
}
// Bounded wait: false (after raising the abort flag and the error word) if
// the phase does not complete in ~2 s, or if the CTA already aborted.
template <uint32_t kHintNs = kSuspendNs>
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abortFlag,
                                          ViDeviceState *st) {
    if (mbar_try_wait<kHintNs>(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait<kHintNs>(bar, parity)) return true;
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
// Bulk prefetch into L2 of `bytes` (a multiple of 16) at a 16-byte aligned p.
__device__ __forceinline__ void prefetch_l2_bytes(const void *p, unsigned bytes) {
    if (bytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// What a lane holds for one slice: the slice's first record and run counts
// (n0 runs, n1 of them with a second record, n2 with a third), the level-0
// records of its runs lane + 32 i (i < kSteps, those that exist) and the
// level-1 and level-2 records of run `lane` (when it has them).
struct SliceRegs {
    uint2 r[kSteps];
    uint2 r1, r2;
    unsigned start, n0, n1, n2;
};
// hdr = {first record, n0, n1, n2} of the slice.
__device__ __forceinline__ void load_slice(SliceRegs &g, const uint2 *__restrict__ rec, uint4 hdr, unsigned lane) {
    g.start = hdr.x;
    g.n0 = hdr.y;
    g.n1 = hdr.z;
    g.n2 = hdr.w;
    const uint2 *p = rec + hdr.x + lane;
    const int c = (int)hdr.y - (int)lane;
#pragma unroll
    for (int i = 0; i < kSteps; i++)
        if (c > 32 * i) g.r[i] = __ldg(p + 32 * i);
    if (lane < hdr.z) g.r1 = __ldg(p + hdr.y);
    if (lane < hdr.w) g.r2 = __ldg(p + hdr.y + hdr.z);
}

// V[s'] of a record: its low half is the byte offset of s' in the tile.
__device__ __forceinline__ float tile_value(const float *vtile, unsigned x) {
    return *reinterpret_cast<const float *>(reinterpret_cast<const char *>(vtile) + (x & 0xFFFFu));
}

// part[row] += fl(gamma*T) * V[s'] for one record.
__device__ __forceinline__ void apply_record(uint2 r, const float *vtile, float *part) {
    part[r.x >> 16] = fadd(part[r.x >> 16], fmul(__uint_as_float(r.y), tile_value(vtile, r.x)));
}

// Records of run j from level 3 on (run j has at least three). Only the rare
// runs of four or more records read level counts.
__device__ __forceinline__ void apply_levels_from3(const SliceRegs &g, unsigned j, const uint2 *__restrict__ rec,
                                                   const unsigned *__restrict__ levelCnt, unsigned L,
                                                   unsigned slice, const float *vtile, float *part) {
    unsigned base = g.n0 + g.n1 + g.n2;
    for (unsigned lv = 3; lv < L; lv++) {
        const unsigned nq = __ldg(levelCnt + (size_t)slice * L + lv);
        if (j >= nq) break;
        apply_record(__ldg(rec + g.start + base + j), vtile, part);
        base += nq;
    }
}

// One slice. The level-0 records a lane holds belong to distinct runs, hence
// distinct rows, and the level-1 and level-2 records of run `lane` to the
// row of its level-0 record r[0]: all their shared-memory reads are issued
// before any write, and the row of r[0] takes its two or three products in
// list order in registers. Then, each in list order after the records
// before it: the level-0 records of runs past 32 kSteps, the further records
// of run `lane`, and the long runs past 32 (rare; records read from L2).
// The plan guarantees every record's row and offset lie inside the block's
// rows and the tile.
__device__ __forceinline__ void apply_slice(const SliceRegs &g, const uint2 *__restrict__ rec,
                                            const unsigned *__restrict__ levelCnt, unsigned L, unsigned slice,
                                            const float *vtile, float *part, unsigned lane) {
    const int c = (int)g.n0 - (int)lane;
    const bool h1 = lane < g.n1, h2 = lane < g.n2;
    float q[kSteps], v[kSteps], v1 = 0.0f, v2 = 0.0f;  // q[i], v[i] are read only where written
#pragma unroll
    for (int i = 0; i < kSteps; i++) {
        if (c > 32 * i) {
            v[i] = tile_value(vtile, g.r[i].x);
            q[i] = part[g.r[i].x >> 16];
        }
    }
    if (h1) v1 = tile_value(vtile, g.r1.x);
    if (h2) v2 = tile_value(vtile, g.r2.x);
#pragma unroll
    for (int i = 0; i < kSteps; i++)
        if (c > 32 * i) q[i] = fadd(q[i], fmul(__uint_as_float(g.r[i].y), v[i]));
    if (h1) q[0] = fadd(q[0], fmul(__uint_as_float(g.r1.y), v1));
    if (h2) q[0] = fadd(q[0], fmul(__uint_as_float(g.r2.y), v2));
#pragma unroll
    for (int i = 0; i < kSteps; i++)
        if (c > 32 * i) part[g.r[i].x >> 16] = q[i];
    if (c > 32 * kSteps)
        for (unsigned j = lane + 32u * kSteps; j < g.n0; j += 32u) apply_record(__ldg(rec + g.start + j), vtile, part);
    if (h2 && L > 3) apply_levels_from3(g, lane, rec, levelCnt, L, slice, vtile, part);
    if (g.n1 > 32u)
        for (unsigned j = lane + 32u; j < g.n1; j += 32u) {
            apply_record(__ldg(rec + g.start + g.n0 + j), vtile, part);
            if (j < g.n2) {
                apply_record(__ldg(rec + g.start + g.n0 + g.n1 + j), vtile, part);
                apply_levels_from3(g, j, rec, levelCnt, L, slice, vtile, part);
            }
        }
}

// One tile of a row warp: load the slice kDepth tiles ahead (and the header
// after it), wait for the V tile, apply the current slice, release the
// buffer.
__device__ __forceinline__ bool row_warp_tile(unsigned t, unsigned T, const SliceRegs &cur, SliceRegs &ahead,
                                              uint4 &hNext, unsigned sl0, const uint2 *__restrict__ rec,
                                              const uint4 *__restrict__ sliceHdr,
                                              const unsigned *__restrict__ levelCnt, unsigned L, const float *vt,
                                              unsigned Vt, float *part, uint64_t *bars, unsigned &sg, unsigned &ph,
                                              volatile int *abortFlag, ViDeviceState *st, unsigned lane) {
    if (t + kDepth < T) {
        load_slice(ahead, rec, hNext, lane);
        // Past the block's last tile this reads the next block's header (or
        // the zeroed padding after the last slice): loaded, never used.
        hNext = __ldg(sliceHdr + sl0 + (t + kDepth + 1) * kRowWarps);
    }
    if (!mbar_wait(smem_addr(&bars[sg]), ph, abortFlag, st)) return false;
    apply_slice(cur, rec, levelCnt, L, sl0 + t * kRowWarps, vt + (size_t)sg * Vt, part, lane);
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_addr(&bars[kStages + sg]));
    if (++sg == kStages) { sg = 0; ph ^= 1u; }
    return true;
}

// A row warp's pass over the block's T tiles. Slice (blk, t) of the warp is
// sl0 + t * kRowWarps. The records of slice t + kDepth are loaded while
// slice t is applied: kDepth + 1 register sets rotate roles, indexed by
// compile-time constants in the unrolled loop, so nothing is copied.
__device__ __forceinline__ bool row_warp_pass(unsigned T, unsigned sl0, const uint2 *__restrict__ rec,
                                              const uint4 *__restrict__ sliceHdr,
                                              const unsigned *__restrict__ levelCnt, unsigned L, const float *vt,
                                              unsigned Vt, float *part, uint64_t *bars, unsigned &sg, unsigned &ph,
                                              volatile int *abortFlag, ViDeviceState *st, unsigned lane) {
    SliceRegs g[kDepth + 1];
#pragma unroll
    for (unsigned u = 0; u <= kDepth; u++) g[u] = SliceRegs{};
#pragma unroll
    for (unsigned u = 0; u < kDepth; u++)
        if (u < T) load_slice(g[u], rec, __ldg(sliceHdr + sl0 + u * kRowWarps), lane);
    uint4 hNext = __ldg(sliceHdr + sl0 + kDepth * kRowWarps);  // padded past the last slice
    for (unsigned t = 0; t < T; t += kDepth + 1) {
#pragma unroll
        for (unsigned u = 0; u <= kDepth; u++) {
            if (t + u >= T) return true;
            if (!row_warp_tile(t + u, T, g[u], g[(u + kDepth) % (kDepth + 1)], hNext, sl0, rec, sliceHdr, levelCnt,
                               L, vt, Vt, part, bars, sg, ph, abortFlag, st, lane))
                return false;
        }
    }
    return true;
}

// Action scan of state i of the block for m = M, a power of two up to 32:
// the thread reads Q(i, .) starting at action rot, so that the 32 lanes of a
// warp (consecutive states) hit 32 distinct banks, rotates the values back
// into action order in registers (log2 M select stages), and scans them as
// mdp_vi_cpu.cpp:55-58 does (first strict maximum).
template <unsigned M>
__device__ __forceinline__ void scan_state_pow2(const float *part, unsigned i, float &best, unsigned &besta) {
    constexpr unsigned LG = M >= 32 ? 5 : M >= 16 ? 4 : M >= 8 ? 3 : M >= 4 ? 2 : M >= 2 ? 1 : 0;
    const unsigned rot = (i >> (5 - LG)) & (M - 1);
    const float *qv = part + (size_t)i * M;
    float q[M];
#pragma unroll
    for (unsigned k = 0; k < M; k++) q[k] = qv[(k + rot) & (M - 1)];  // q[k] = Q(i, k + rot)
#pragma unroll
    for (int b = 0; b < (int)LG; b++) {
        // Rotate right by 2^b when bit b of rot is set.
        const bool on = (rot >> b) & 1u;
        float r[M];
#pragma unroll
        for (unsigned k = 0; k < M; k++) r[k] = on ? q[(k + M - (1u << b)) & (M - 1)] : q[k];
#pragma unroll
        for (unsigned k = 0; k < M; k++) q[k] = r[k];
    }
    best = q[0];
    besta = 0;
#pragma unroll
    for (unsigned a = 1; a < M; a++)
        if (q[a] > best) { best = q[a]; besta = a; }
}

// Largest |Vp - V| over a thread's states, as (Vp, V) of the largest: the
// rounded float difference orders the exact ones except on ties, which are
// settled in double (a zero difference is exact). NaN differences are
// skipped, as fmax skips them.
struct ResidualMax {
    float d = 0.0f, a = 0.0f, b = 0.0f;
    __device__ __forceinline__ void add(float x, float y) {
        const float e = fabsf(__fsub_rn(x, y));
        if (e > d || (e == d && e != 0.0f && fabs((double)x - (double)y) > fabs((double)a - (double)b))) {
            d = e;
            a = x;
            b = y;
        }
    }
    __device__ __forceinline__ double value() const { return fabs((double)a - (double)b); }
};

// Action scan of the block's nsb states by the row-warp threads (rt of
// kRowWarps * 32, one state each in turn): Vp, pi and the largest |Vp - V|.
// The V of kBatch states is loaded before they are scanned.
template <unsigned M>
__device__ __forceinline__ double scan_block_m(const float *part, unsigned nsb, unsigned m, unsigned s0,
                                               const float *__restrict__ V, float *__restrict__ Vp,
                                               unsigned *__restrict__ pi, unsigned rt, double local) {
    constexpr unsigned kStride = kRowWarps * 32, kBatch = M >= 32 ? 2 : M >= 16 ? 4 : 8;
    ResidualMax res;
    for (unsigned i0 = rt; i0 < nsb; i0 += kStride * kBatch) {
        float vOld[kBatch];
#pragma unroll
        for (unsigned b = 0; b < kBatch; b++) {
            const unsigned i = i0 + b * kStride;
            vOld[b] = i < nsb ? __ldg(V + s0 + i) : 0.0f;
        }
#pragma unroll
        for (unsigned b = 0; b < kBatch; b++) {
            const unsigned i = i0 + b * kStride;
            if (i >= nsb) break;
            float best;
            unsigned besta;
            if constexpr (M != 0) {
                scan_state_pow2<M>(part, i, best, besta);
            } else {
                // Any other m: mdp_vi_cpu.cpp:55-58 as written (lowest action on ties).
                const float *qv = part + (size_t)i * m;
                best = qv[0];
                besta = 0;
                for (unsigned a = 1; a < m; a++)
                    if (qv[a] > best) { best = qv[a]; besta = a; }
            }
            Vp[s0 + i] = best;
            pi[s0 + i] = besta;
            res.add(best, vOld[b]);
        }
    }
    return fmax(local, res.value());
}

__device__ __forceinline__ double scan_block(const float *part, unsigned nsb, unsigned m, unsigned s0,
                                             const float *__restrict__ V, float *__restrict__ Vp,
                                             unsigned *__restrict__ pi, unsigned rt, double local) {
    switch (m) {
        case 1: return scan_block_m<1>(part, nsb, m, s0, V, Vp, pi, rt, local);
        case 2: return scan_block_m<2>(part, nsb, m, s0, V, Vp, pi, rt, local);
        case 4: return scan_block_m<4>(part, nsb, m, s0, V, Vp, pi, rt, local);
        case 8: return scan_block_m<8>(part, nsb, m, s0, V, Vp, pi, rt, local);
        case 16: return scan_block_m<16>(part, nsb, m, s0, V, Vp, pi, rt, local);
        case 32: return scan_block_m<32>(part, nsb, m, s0, V, Vp, pi, rt, local);
        default: return scan_block_m<0>(part, nsb, m, s0, V, Vp, pi, rt, local);
    }
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
    // bars: full[kStages], empty[kStages], qReady, qFree; then two flags.
    const uint32_t qReady = smem_addr(&bars[2 * kStages]), qFree = smem_addr(&bars[2 * kStages + 1]);
    volatile int *abortFlag = reinterpret_cast<volatile int *>(bars + 2 * kStages + 2);
    volatile int *rowAbort = abortFlag + 1;
    const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (unsigned s = 0; s < kStages; s++) {
            mbar_init(smem_addr(&bars[s]), 1);                 // full: the staging lane's arrival + bytes
            mbar_init(smem_addr(&bars[kStages + s]), kRowWarps);  // empty: one arrival per row warp
        }
        mbar_init(qReady, 1);          // the block's R in Q: the staging lane's arrival + bytes
        mbar_init(qFree, kRowWarps);   // the block's scan done: one arrival per row warp
        *abortFlag = 0;
        *rowAbort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    double local = 0.0;
    if (warp == kRowWarps) {
        // ---- staging warp (lane 0): per block, R into Q once the previous
        // block's scan released it (one bulk copy; the next block's R is
        // prefetched into L2), and V tile after tile into the ring, which
        // runs on across block boundaries; records into L2 kAhead tiles
        // ahead of the row warps.
        if (lane == 0) {
            unsigned lastPar[kStages];  // parity of the last copy issued per stage (2: none)
#pragma unroll
            for (unsigned s = 0; s < kStages; s++) lastPar[s] = 2u;
            unsigned rLastPar = 2u;     // parity of the last R copy issued (2: none)
            unsigned sg = 0, ph = 0, it = 0;
            bool ok = true;
            for (unsigned blk = blockIdx.x; ok && blk < blocks; blk += gridDim.x, it++) {
                const unsigned s0 = blk * Sb, nsb = min(Sb, n - s0), rows = nsb * m;
                const size_t c0 = (size_t)blk * T;
                if (it == 0)
                    prefetch_l2(rec, __ldg(sliceStart + c0 * kRowWarps),
                                __ldg(sliceStart + (c0 + min(T, kAhead)) * kRowWarps));
                // R goes in after the first kStages tiles of the block were
                // issued (their slots were freed by the previous block's
                // last tiles, before its scan); the CTA's first block copies
                // it before its first V tiles.
                const unsigned rAt = it == 0 ? 0u : min(T, kStages);
                for (unsigned t = 0; t <= T; t++) {
                    if (t == rAt) {
                        if (it > 0 && !mbar_wait<0>(qFree, (it - 1) & 1u, abortFlag, st)) { ok = false; break; }
                        const float *src = R + (size_t)s0 * m;
                        const unsigned body = rows & ~3u;
                        for (unsigned k = body; k < rows; k++) part[k] = __ldg(src + k);
                        mbar_expect_tx(qReady, body * 4u);
                        if (body) bulk_copy(smem_addr(part), src, body * 4u, qReady);
                        rLastPar = it & 1u;
                        if (blk + gridDim.x < blocks) {
                            const unsigned nb = blk + gridDim.x;
                            const unsigned nrows = min(Sb, n - nb * Sb) * m;
                            prefetch_l2_bytes(R + (size_t)nb * Sb * m, (nrows * 4u) & ~15u);
                        }
                    }
                    if (t == T) break;
                    if (!mbar_wait(smem_addr(&bars[kStages + sg]), ph ^ 1u, abortFlag, st)) { ok = false; break; }
                    const unsigned base = t * Vt, cnt = min(Vt, n - base);
                    const unsigned body = cnt & ~3u;
                    float *dst = vt + (size_t)sg * Vt;
                    for (unsigned k = body; k < cnt; k++) dst[k] = __ldg(V + base + k);  // tail of the last tile
                    const uint32_t fb = smem_addr(&bars[sg]);
                    mbar_expect_tx(fb, body * 4u);
                    if (body) bulk_copy(smem_addr(dst), V + base, body * 4u, fb);
                    lastPar[sg] = ph;
                    {
                        const unsigned ahead = t + kAhead;
                        size_t pc = ~(size_t)0;
                        if (ahead < T) pc = c0 + ahead;
                        else if (blk + gridDim.x < blocks && ahead - T < T) pc = (size_t)(blk + gridDim.x) * T + (ahead - T);
                        if (pc != ~(size_t)0)
                            prefetch_l2(rec, __ldg(sliceStart + pc * kRowWarps), __ldg(sliceStart + (pc + 1) * kRowWarps));
                    }
                    if (++sg == kStages) { sg = 0; ph ^= 1u; }
                }
            }
            if (*abortFlag) {
                // Let the copies in flight land before the CTA exits
                // (bounded): the last issue on each barrier completes the
                // phase of the parity recorded.
                for (unsigned s = 0; s < kStages; s++) {
                    if (lastPar[s] > 1u) continue;
                    const long long t0 = clock64();
                    while (!mbar_try_wait<0>(smem_addr(&bars[s]), lastPar[s]) && clock64() - t0 < kWaitCycles) {
                    }
                }
                if (rLastPar <= 1u) {
                    const long long t0 = clock64();
                    while (!mbar_try_wait<0>(qReady, rLastPar) && clock64() - t0 < kWaitCycles) {
                    }
                }
            }
        }
    } else {
        // ---- row warps ----
        // Per block: wait for R in Q, apply the block's slices tile after
        // tile, meet at a named barrier, scan, release Q. The decision to
        // stop is taken from rowAbort, which only row warps write and only
        // before the barrier, so every row warp takes it alike.
        unsigned sg = 0, ph = 0, it = 0;
        for (unsigned blk = blockIdx.x; blk < blocks; blk += gridDim.x, it++) {
            const unsigned s0 = blk * Sb, nsb = min(Sb, n - s0);
            bool ok = mbar_wait<0>(qReady, it & 1u, abortFlag, st);
            if (ok)
                ok = row_warp_pass(T, (unsigned)((size_t)blk * T * kRowWarps) + warp, rec, sliceHdr, levelCnt, L, vt,
                                   Vt, part, bars, sg, ph, abortFlag, st, lane);
            if (!ok && lane == 0) *rowAbort = 1;
            asm volatile("bar.sync 1, %0;" ::"r"(kRowWarps * 32) : "memory");
            if (*rowAbort) break;
            local = scan_block(part, nsb, m, s0, V, Vp, pi, warp * 32 + lane, local);
            // Q is next written by the bulk copy (async proxy).
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(qFree);
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
            rec[base + j] = make_uint2((rowLocal << 16) | ((sp - t * g.Vt) * 4u), __float_as_uint(fmul(g.gamma, Tr[l0 + q])));
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
    const size_t reserve = 1024;  // static shared memory of the residual reduction, with room to spare
    // Waves of blocks (rounds of Sb-state blocks over the SMs) a tile size
    // leaves room for: the V ring and Q share the CTA's shared memory.
    auto waves_for = [&](unsigned vt) -> unsigned {
        const size_t fx = (size_t)kStages * vt * 4 + 16 + kBarrierBytes;
        if ((size_t)optin < fx + reserve + (size_t)m * 4) return ~0u;
        const unsigned rows = (unsigned)std::min<size_t>(((size_t)optin - fx - reserve) / 4, kMaxRows);
        const unsigned sb = rows / m;
        return sb == 0 ? ~0u : (unsigned)ceil_div(n, (unsigned long long)sms * sb);
    };
    const unsigned setting = g_tile_states.load();
    unsigned Vt = setting;
    if (Vt == 0) {
        // Default: the largest tile in [kDefaultTileStates, kMaxDefaultTileStates]
        // (steps of 256 states) that needs no more waves than the smallest:
        // fewer, longer tiles cut the per-slice work, another wave re-reads V.
        Vt = kDefaultTileStates;
        const unsigned w0 = waves_for(kDefaultTileStates);
        for (unsigned vt = kDefaultTileStates + 256; vt <= kMaxDefaultTileStates; vt += 256)
            if (waves_for(vt) <= w0) Vt = vt;
    }
    Vt = std::min<unsigned>(Vt, (unsigned)round_up(n, 4));
    const unsigned tiles = ceil_div(n, Vt);
    const size_t fixed = (size_t)kStages * Vt * 4 + 16 + kBarrierBytes;
    if ((size_t)optin < fixed + reserve + (size_t)m * 4) return NOVA_SUCCESS;
    const unsigned rowsMax = (unsigned)std::min<size_t>(((size_t)optin - fixed - reserve) / 4, kMaxRows);
    const unsigned SbMax = rowsMax / m;
    if (SbMax == 0) return NOVA_SUCCESS;
    const unsigned waves = ceil_div(n, (unsigned long long)sms * SbMax);
    // Sb * m a multiple of 4, so that every block's R starts 16-byte aligned
    // (one bulk copy per block).
    const unsigned qAlign = (m % 4u == 0u) ? 1u : (m % 2u == 0u) ? 2u : 4u;
    unsigned Sb = (unsigned)round_up(ceil_div(n, (unsigned long long)sms * waves), qAlign);
    if (Sb > SbMax) Sb = SbMax / qAlign * qAlign;
    if (Sb == 0) return NOVA_SUCCESS;
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
    // Headers, with (kDepth + 1) * kRowWarps zeroed ones after the last slice
    // for the row warps' unconditional look-ahead loads.
    const size_t hdrPad = (size_t)(kDepth + 1) * kRowWarps;
    if (rc == NOVA_SUCCESS && !try_alloc(&plan->sliceHdr, nSlices + hdrPad)) rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS &&
            cudaMemsetAsync(plan->sliceHdr + nSlices, 0, hdrPad * sizeof(uint4), stream) != cudaSuccess) {
        cudaGetLastError();
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
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
        // (A record's byte offset in its tile, below 4 * 16384, fits its 16-bit field.)
        NOVA_ERR("mdp_vi_set_tiling_gpu", "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    nova_gb300::g_mode.store(mode);
    nova_gb300::g_tile_states.store(tileStates);
    return NOVA_SUCCESS;
}
