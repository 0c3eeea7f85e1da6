// nova-gb300: column-tiled Bellman sweep for large sparse MDPs.
//
// The per-row sweep (mdp_vi.cu) gathers V[S(s,a,l)] straight from L2: at
// n = 2^20, m = 8, ns = 16 that is 134M random 4-byte requests per sweep,
// and L1/L2 request throughput, not HBM, bounds it. This sweep turns the
// gathers into shared-memory reads:
//
//   * Source states are cut into blocks of Sb states (one CTA at a time per
//     block; its m*Sb partial sums Q(s,a) live in shared memory, seeded with
//     R(s,a)). Successor states are cut into tiles of Vt states; the CTA
//     stages V one tile at a time (cp.async, double-buffered) and adds the
//     products of the successors that fall in that tile.
//   * The plan regroups the successor entries once per solver: one 8-byte
//     record {row << 16 | offset in tile, fl(gamma * T)} per entry (the
//     reference's first rounding, done once). Within a block the
//     m*Sb rows are split into equal ranges, one per warp, so a row is
//     only ever touched by one warp. A row's successors that fall in one tile
//     form a run (they are consecutive in the row's list); the q-th record of
//     every run goes to level q. The records of (block, tile, warp) are
//     stored level after level, so within a level every row appears at most
//     once and lanes add to their rows' partial sums without conflicts, and
//     level q is applied before level q+1, which keeps each row's products in
//     list order. Records stream from HBM exactly once per sweep (the same 8
//     bytes per entry as S and T).
//
// Order of operations: the reference computes Q = R(s,a), then for each
// successor in list order Q += (gamma * T) * V[s'] (mdp_vi_cpu.cpp:45-52).
// When every row's successors are listed in ascending state order, tile
// order is list order, so this sweep performs the same roundings in the same
// order and its results are bit-identical. The plan builder checks that;
// models with unsorted rows keep the per-row sweep.

#include "vi.h"

#include <algorithm>
#include <atomic>

#include <nova/nova_gb300.h>

using nova::MDP;

namespace nova_gb300 {

namespace {

constexpr unsigned kThreads = 1024;
constexpr unsigned kWarps = kThreads / 32;     // row ranges (and level slices) per block
constexpr int kPairGroups = 4;             // groups of 64 records (32 pairs) prefetched per warp
constexpr unsigned kMaxRows = 65535u;       // rows of one block (16-bit row field)
constexpr unsigned kDefaultTileStates = 10240u;
constexpr unsigned long long kAutoMinEntries = 1ull << 22;

std::atomic<unsigned> g_mode{NOVA_VI_TILING_AUTO};
std::atomic<unsigned> g_tile_states{0};
std::atomic<unsigned> g_last_status{0};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Stage V[t*Vt, min(n, (t+1)*Vt)) into dst: 16-byte cp.async for the
// aligned body, plain loads for the tail of the last tile.
__device__ __forceinline__ void stage_tile(float *dst, const float *__restrict__ V, unsigned n, unsigned t,
                                           unsigned Vt) {
    const unsigned base = t * Vt;
    const unsigned cnt = min(Vt, n - base);
    const unsigned c4 = cnt >> 2;
    for (unsigned i = threadIdx.x; i < c4; i += blockDim.x) cp_async16(dst + 4 * i, V + base + 4 * i);
    for (unsigned i = (c4 << 2) + threadIdx.x; i < cnt; i += blockDim.x) dst[i] = V[base + i];
    cp_async_commit();
}

// Records of one warp slice are read as 16-byte pairs: pair j of the slice
// holds records 2j and 2j+1 counted from a0, the slice start rounded down
// to an even record (the record array has one spare record at its end).
__device__ __forceinline__ void load_pairs(uint4 (&buf)[kPairGroups], const uint4 *__restrict__ rec2, unsigned a0,
                                           unsigned b1, unsigned lane) {
#pragma unroll
    for (int k = 0; k < kPairGroups; k++) {
        const unsigned j = (a0 >> 1) + 32u * k + lane;
        buf[k] = 2u * j < b1 ? __ldg(rec2 + j) : make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
    }
}

// Apply one pair-group: records [g0, g0 + 64) of this warp's slice, lane l
// holding records g0 + 2l and g0 + 2l + 1; records outside [b0, b1) and
// padding records are skipped. The plan keeps two records of one row at
// least 64 positions apart, so the rows of a pair-group are distinct; groups
// run in slice order, which is each row's successor order.
__device__ __forceinline__ void apply_pairs(uint4 r, unsigned g0, unsigned b0, unsigned b1, unsigned lane,
                                            const float *vtile, unsigned tileLen, float *part,
                                            unsigned rows) {
    const unsigned p0 = g0 + 2u * lane, p1 = p0 + 1u;
    const unsigned row0 = r.x >> 16, off0 = r.x & 0xFFFFu;
    const unsigned row1 = r.z >> 16, off1 = r.z & 0xFFFFu;
    if (p0 >= b0 && p0 < b1 && row0 < rows && off0 < tileLen)
        part[row0] = fadd(part[row0], fmul(__uint_as_float(r.y), vtile[off0]));
    if (p1 >= b0 && p1 < b1 && row1 < rows && off1 < tileLen)
        part[row1] = fadd(part[row1], fmul(__uint_as_float(r.w), vtile[off1]));
    __syncwarp();
}

__global__ void __launch_bounds__(kThreads, 1) bellman_tiled_kernel(
        unsigned n, unsigned m, unsigned Vt, unsigned T, unsigned Sb, unsigned blocks,
        const uint2 *__restrict__ rec, const unsigned *__restrict__ sliceStart, const float *__restrict__ R,
        const float *__restrict__ V, float *__restrict__ Vp, unsigned *__restrict__ pi, ViDeviceState *st,
        double tol, int early_exit) {
    if (early_exit && *(volatile unsigned *)&st->converged) return;  // uniform across the grid
    extern __shared__ __align__(16) unsigned char smem[];
    float *vt = reinterpret_cast<float *>(smem);            // [2][Vt]
    float *part = vt + 2 * (size_t)Vt;                      // [Sb*m]
    const uint4 *rec2 = reinterpret_cast<const uint4 *>(rec);
    const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    double local = 0.0;
    for (unsigned blk = blockIdx.x; blk < blocks; blk += gridDim.x) {
        const unsigned s0 = blk * Sb;
        const unsigned nsb = min(Sb, n - s0);
        const unsigned rows = nsb * m;
        for (unsigned i = tid; i < rows; i += blockDim.x) part[i] = __ldg(R + (size_t)s0 * m + i);
        // Slice (block, tile, warp) is sliceStart[(blk*T + t)*kWarps + warp] ..
        // sliceStart[... + 1]; lanes 0 and 1 hold the two bounds.
        const size_t sub0 = (size_t)blk * T * kWarps + warp;
        unsigned bdCur = lane < 2 ? __ldg(sliceStart + sub0 + lane) : 0u;
        unsigned bdNext = (T > 1 && lane < 2) ? __ldg(sliceStart + sub0 + kWarps + lane) : 0u;
        stage_tile(vt, V, n, 0, Vt);
        uint4 cur[kPairGroups], nxt[kPairGroups];
#pragma unroll
        for (int k = 0; k < kPairGroups; k++) nxt[k] = make_uint4(0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u);
        load_pairs(cur, rec2, __shfl_sync(0xffffffffu, bdCur, 0) & ~1u, __shfl_sync(0xffffffffu, bdCur, 1), lane);
        cp_async_wait_all();
        __syncthreads();
        for (unsigned t = 0; t < T; t++) {
            const float *vcur = vt + (size_t)(t & 1) * Vt;
            unsigned bdNext2 = 0u;
            if (t + 1 < T) {
                // The other buffer held tile t-1; every warp passed the
                // barrier that ended tile t-1, so it is free.
                stage_tile(vt + (size_t)((t + 1) & 1) * Vt, V, n, t + 1, Vt);
                load_pairs(nxt, rec2, __shfl_sync(0xffffffffu, bdNext, 0) & ~1u,
                           __shfl_sync(0xffffffffu, bdNext, 1), lane);
                if (t + 2 < T && lane < 2) bdNext2 = __ldg(sliceStart + sub0 + (size_t)(t + 2) * kWarps + lane);
            }
            const unsigned b0 = __shfl_sync(0xffffffffu, bdCur, 0), b1 = __shfl_sync(0xffffffffu, bdCur, 1);
            const unsigned a0 = b0 & ~1u;
            const unsigned tileLen = min(Vt, n - t * Vt);
            for (unsigned c0 = a0; c0 < b1; c0 += 64u * kPairGroups) {
                if (c0 != a0) load_pairs(cur, rec2, c0, b1, lane);
#pragma unroll
                for (int k = 0; k < kPairGroups; k++) {
                    const unsigned g0 = c0 + 64u * k;
                    if (g0 < b1) apply_pairs(cur[k], g0, b0, b1, lane, vcur, tileLen, part, rows);
                }
            }
            cp_async_wait_all();
            __syncthreads();
#pragma unroll
            for (int k = 0; k < kPairGroups; k++) cur[k] = nxt[k];
            bdCur = bdNext;
            bdNext = bdNext2;
        }
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
    unsigned n, m, ns, Vt, T, Sb, rowsPerWarp, L;
    float gamma;
    __device__ __forceinline__ size_t sub(unsigned blk, unsigned t, unsigned rowLocal) const {
        return (((size_t)blk * T + t) * kWarps + rowLocal / rowsPerWarp) * L;
    }
};

// Records per (block, tile, warp, level) sub-bin.
__global__ void vi_plan_count_kernel(PlanGeometry g, const int *__restrict__ S, unsigned *counts) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)g.n * g.m) return;
    const unsigned blk = (unsigned)(row / g.m) / g.Sb;
    const unsigned rowLocal = (unsigned)(row - (unsigned long long)blk * g.Sb * g.m);
    const int *Sr = S + row * g.ns;
    unsigned runTile = 0xFFFFFFFFu, q = 0;
    for (unsigned l = 0; l < g.ns; l++) {
        const int sp = Sr[l];
        if (sp < 0) break;
        const unsigned t = (unsigned)sp / g.Vt;
        q = t == runTile ? q + 1 : 0;
        runTile = t;
        atomicAdd(counts + g.sub(blk, t, rowLocal) + q, 1u);
    }
}

// Write every record to its sub-bin. One thread per (block, warp) owns all
// sub-bins of that warp's row range and walks its rows in order, so each
// sub-bin lists its rows in ascending order (fewer shared-memory bank
// conflicts on the partial sums) and the plan does not depend on timing.
__global__ void vi_plan_fill_kernel(PlanGeometry g, unsigned blocks, const int *__restrict__ S,
                                    const float *__restrict__ Tm, const unsigned *__restrict__ start,
                                    unsigned *cursor, uint2 *rec) {
    const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned blk = idx / kWarps, w = idx % kWarps;
    if (blk >= blocks) return;
    const unsigned nsb = min(g.Sb, g.n - blk * g.Sb);
    const unsigned rowsBlk = nsb * g.m;
    const unsigned r0 = w * g.rowsPerWarp, r1 = min(rowsBlk, r0 + g.rowsPerWarp);
    for (unsigned rowLocal = r0; rowLocal < r1; rowLocal++) {
        const unsigned long long row = (unsigned long long)blk * g.Sb * g.m + rowLocal;
        const int *Sr = S + row * g.ns;
        const float *Tr = Tm + row * g.ns;
        unsigned runTile = 0xFFFFFFFFu, q = 0;
        for (unsigned l = 0; l < g.ns; l++) {
            const int sp = Sr[l];
            if (sp < 0) break;
            const unsigned t = (unsigned)sp / g.Vt;
            q = t == runTile ? q + 1 : 0;
            runTile = t;
            const size_t sb = g.sub(blk, t, rowLocal) + q;
            const unsigned c = cursor[sb];
            cursor[sb] = c + 1;
            rec[start[sb] + c] =
                make_uint2((rowLocal << 16) | ((unsigned)sp - t * g.Vt), __float_as_uint(fmul(g.gamma, Tr[l])));
        }
    }
}

// Final layout. Slice sl = (block, tile, warp) holds levels 0..L-1, each
// sorted by row. The run length of a row (the number of levels it appears
// in) is found from the deepest level up; the final slice lists, level after
// level, the rows of that level ordered by (run length descending, row), so
// level q+1 is a prefix-aligned continuation of level q, and each level
// after the first starts at least 64 records after the previous one (padding
// records in between). Two records of one row are then always at least 64
// positions apart: any 64 consecutive records have distinct rows.
__global__ void vi_plan_len_kernel(unsigned nSlices, unsigned L, const unsigned *__restrict__ ls,
                                   const uint2 *__restrict__ recL, unsigned char *__restrict__ len) {
    const unsigned sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nSlices) return;
    const size_t base = (size_t)sl * L;
    for (int q = (int)L - 1; q >= 0; q--) {
        const unsigned e0 = ls[base + q], e1 = ls[base + q + 1];
        if (q == (int)L - 1) {
            for (unsigned e = e0; e < e1; e++) len[e] = (unsigned char)L;
            continue;
        }
        unsigned p = e1;  // level q+1 starts where level q ends
        const unsigned p1 = ls[base + q + 2];
        for (unsigned e = e0; e < e1; e++) {
            const unsigned row = recL[e].x >> 16;
            while (p < p1 && (recL[p].x >> 16) < row) p++;
            len[e] = (p < p1 && (recL[p].x >> 16) == row) ? len[p] : (unsigned char)(q + 1);
        }
    }
}

__device__ __forceinline__ unsigned slice_levels(const unsigned *ls, size_t base, unsigned L) {
    unsigned q = 0;
    while (q < L && ls[base + q + 1] > ls[base + q]) q++;
    return q;
}

__global__ void vi_plan_size_kernel(unsigned nSlices, unsigned L, const unsigned *__restrict__ ls,
                                    unsigned *__restrict__ size) {
    const unsigned sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nSlices) return;
    const size_t base = (size_t)sl * L;
    const unsigned Ls = slice_levels(ls, base, L);
    unsigned pos = 0;
    for (unsigned q = 0; q < Ls; q++) {
        const unsigned start = pos;
        pos += ls[base + q + 1] - ls[base + q];
        if (q + 1 < Ls) pos = max(pos, start + 64u);
    }
    size[sl] = pos;
}

__global__ void vi_plan_order_kernel(unsigned nSlices, unsigned L, const unsigned *__restrict__ ls,
                                     const uint2 *__restrict__ recL, const unsigned char *__restrict__ len,
                                     const unsigned *__restrict__ sliceStart, uint2 *__restrict__ rec) {
    const unsigned sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= nSlices) return;
    const size_t base = (size_t)sl * L;
    const unsigned Ls = slice_levels(ls, base, L);
    uint2 *out = rec + sliceStart[sl];
    unsigned pos = 0;
    for (unsigned q = 0; q < Ls; q++) {
        const unsigned start = pos;
        const unsigned e0 = ls[base + q], e1 = ls[base + q + 1];
        for (unsigned l = Ls; l > q; l--)
            for (unsigned e = e0; e < e1; e++)
                if (len[e] == l) out[pos++] = recL[e];
        if (q + 1 < Ls) pos = max(pos, start + 64u);  // padding slots keep the sentinel
    }
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
    cudaFree(plan->levelStart);
    cudaFree(plan->sliceStart);
    cudaFree(plan->counts);
    cudaFree(plan->flags);
    plan->rec = nullptr;
    plan->levelStart = plan->sliceStart = plan->counts = plan->flags = nullptr;
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
    const size_t fixed = 2 * (size_t)Vt * 4;
    const size_t reserve = 1024;  // static shared memory of the residual reduction, with room to spare
    if ((size_t)optin < fixed + reserve + (size_t)m * 4) return NOVA_SUCCESS;
    const unsigned rowsMax = (unsigned)std::min<size_t>(((size_t)optin - fixed - reserve) / 4, kMaxRows);
    const unsigned SbMax = rowsMax / m;
    if (SbMax == 0) return NOVA_SUCCESS;
    const unsigned waves = ceil_div(n, (unsigned long long)sms * SbMax);
    const unsigned Sb = ceil_div(n, (unsigned long long)sms * waves);
    const unsigned blocks = ceil_div(n, Sb);
    const size_t smemBytes = fixed + round_up((size_t)Sb * m * 4, 16);

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
    if (hflags[0] != 0 || hflags[1] != 0 || L > 31) {
        release(plan);
        return NOVA_SUCCESS;
    }
    PlanGeometry g{n, m, ns, Vt, tiles, Sb, ceil_div((unsigned long long)Sb * m, kWarps), L, mdp->gamma};
    const unsigned long long nSub = (unsigned long long)blocks * tiles * kWarps * L;
    if (nSub >= (1ull << 32) - 1) { release(plan); return NOVA_SUCCESS; }

    // Pass 2: sub-bin sizes and their exclusive scan.
    if (!try_alloc(&plan->counts, nSub) || !try_alloc(&plan->levelStart, nSub + 1)) {
        release(plan);
        return NOVA_SUCCESS;
    }
    if (cudaMemsetAsync(plan->counts, 0, nSub * sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan counters.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    vi_plan_count_kernel<<<rowBlocks, 256, 0, stream>>>(g, S, plan->counts);
    if ((rc = check_launch(fn, "sweep plan (count)")) != NOVA_SUCCESS) { release(plan); return rc; }
    rc = scan_counts(plan->counts, nSub, plan->levelStart, stream, fn);
    if (rc == NOVA_ERROR_DEVICE_MALLOC) { release(plan); return NOVA_SUCCESS; }
    if (rc != NOVA_SUCCESS) { release(plan); return rc; }
    unsigned total = 0;
    if ((rc = d2h(&total, plan->levelStart + nSub, sizeof(unsigned), fn, "the sweep plan size")) != NOVA_SUCCESS) {
        release(plan);
        return rc;
    }

    // Pass 3: records (one spare at the end: the sweep reads them in pairs).
    if (!try_alloc(&plan->rec, (size_t)total + 1)) { release(plan); return NOVA_SUCCESS; }
    if (cudaMemsetAsync(plan->counts, 0, nSub * sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan cursors.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (cudaMemsetAsync(plan->rec + total, 0xFF, sizeof(uint2), stream) != cudaSuccess) {
        cudaGetLastError();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan records.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    vi_plan_fill_kernel<<<ceil_div((unsigned long long)blocks * kWarps, 128), 128, 0, stream>>>(
        g, blocks, S, T, plan->levelStart, plan->counts, plan->rec);
    if ((rc = check_launch(fn, "sweep plan (fill)")) != NOVA_SUCCESS) { release(plan); return rc; }
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) { release(plan); return rc; }
    cudaFree(plan->counts);
    cudaFree(plan->flags);
    plan->counts = plan->flags = nullptr;

    // Pass 4: the final layout (rows by run length, levels 64 records apart).
    const unsigned nSlices = (unsigned)((unsigned long long)blocks * tiles * kWarps);
    unsigned char *len = nullptr;
    unsigned *sliceSize = nullptr;
    uint2 *rec2 = nullptr;
    if (!try_alloc(&len, (size_t)total + 1) || !try_alloc(&sliceSize, nSlices) ||
            !try_alloc(&plan->sliceStart, (size_t)nSlices + 1)) {
        cudaFree(len);
        cudaFree(sliceSize);
        release(plan);
        return NOVA_SUCCESS;
    }
    const unsigned sliceBlocks = ceil_div(nSlices, 128);
    vi_plan_len_kernel<<<sliceBlocks, 128, 0, stream>>>(nSlices, L, plan->levelStart, plan->rec, len);
    rc = check_launch(fn, "sweep plan (run lengths)");
    if (rc == NOVA_SUCCESS) {
        vi_plan_size_kernel<<<sliceBlocks, 128, 0, stream>>>(nSlices, L, plan->levelStart, sliceSize);
        rc = check_launch(fn, "sweep plan (slice sizes)");
    }
    if (rc == NOVA_SUCCESS) rc = scan_counts(sliceSize, nSlices, plan->sliceStart, stream, fn);
    unsigned total2 = 0;
    if (rc == NOVA_SUCCESS)
        rc = d2h(&total2, plan->sliceStart + nSlices, sizeof(unsigned), fn, "the sweep plan size");
    // Small slices pay a lot of padding; in automatic mode such models keep
    // the per-row sweep.
    if (rc == NOVA_SUCCESS && mode == NOVA_VI_TILING_AUTO && (double)total2 > 1.5 * (double)total)
        rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS && !try_alloc(&rec2, (size_t)total2 + 1)) rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS && cudaMemsetAsync(rec2, 0xFF, ((size_t)total2 + 1) * sizeof(uint2), stream) != cudaSuccess) {
        cudaGetLastError();
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (rc == NOVA_SUCCESS) {
        vi_plan_order_kernel<<<sliceBlocks, 128, 0, stream>>>(nSlices, L, plan->levelStart, plan->rec, len,
                                                              plan->sliceStart, rec2);
        rc = check_launch(fn, "sweep plan (order)");
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    cudaFree(len);
    cudaFree(sliceSize);
    if (rc != NOVA_SUCCESS) {
        cudaFree(rec2);
        release(plan);
        return rc == NOVA_ERROR_DEVICE_MALLOC ? NOVA_SUCCESS : rc;  // kGather
    }
    cudaFree(plan->rec);
    cudaFree(plan->levelStart);
    plan->levelStart = nullptr;
    plan->rec = rec2;
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
        mdp->n, mdp->m, plan->tileStates, plan->tiles, plan->blockStates, plan->blocks, plan->rec,
        plan->sliceStart, R, V, Vp, pi, st, tol, early_exit);
    return check_launch(fn, "Bellman update (tiled)");
}

unsigned vi_last_plan_status() { return g_last_status.load(); }

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
