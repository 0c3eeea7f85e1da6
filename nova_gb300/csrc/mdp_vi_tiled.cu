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
//   * A row's successors inside one tile form a run (consecutive in the
//     row's list). The plan, built once per solver, stores for every chunk
//     (block, tile) the 8-byte records {row << 16 | offset in tile,
//     fl(gamma * T)} (the reference's first rounding, done once) of all its
//     runs, level after level: level q holds the q-th record of every run
//     with more than q records, runs ordered by length (longest first), so
//     run j has its level-q record at position j of level q. Thread k of the
//     CTA applies runs k, k + 1024, ... of the chunk, each run's records in
//     list order into its row's partial sum; the rows of one chunk's runs are
//     distinct, so no two threads touch one partial sum, and the chunks of a
//     block run in tile order with one CTA barrier between tiles. Records
//     stream from HBM exactly once per sweep (the same 8 bytes per entry as S
//     and T): each thread loads its next chunk's records into registers while
//     it applies the current chunk's, and the chunk after that is prefetched
//     into L2 with one bulk prefetch.
//   * Within a chunk the single-record runs are ordered so that a warp's 32
//     runs fall in distinct shared-memory banks: runs are bucketed by the
//     bank of their partial sum (row mod 32), sorted inside each bucket by
//     the distance (tile offset - row) mod 32, and dealt out round-robin over
//     the buckets. A full round is 32 distinct partial-sum banks, and since
//     the k-th runs of the buckets have about the same distance, their V
//     offsets fall in distinct banks too.
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
constexpr int kRunsPerThread = 5;           // level-0 records held in registers per thread and chunk
constexpr unsigned kMaxRows = 65535u;       // rows of one block (16-bit row field)
constexpr unsigned kMaxLevels = 31u;        // longest run of one row inside one tile
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

// Bulk prefetch of a record range into L2 (16-byte aligned; the record
// array has two spare records at its end).
__device__ __forceinline__ void prefetch_l2(const uint2 *rec, unsigned b, unsigned e) {
    if (e <= b) return;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(rec + b) & ~(uintptr_t)15;
    const uintptr_t hi = (reinterpret_cast<uintptr_t>(rec + e) + 15) & ~(uintptr_t)15;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
}

// The records a thread needs for one chunk: level-0 records of its runs
// tid + kThreads * i (i < kRunsPerThread), and the level-1 record of run tid.
struct ChunkRegs {
    uint2 r0[kRunsPerThread];
    uint2 r1;
    unsigned start, n0, n1;
};

__device__ __forceinline__ void load_chunk(ChunkRegs &c, const uint2 *__restrict__ rec,
                                           const unsigned *__restrict__ chunkStart,
                                           const unsigned *__restrict__ levelCnt, unsigned L, size_t chunk,
                                           unsigned tid) {
    c.start = __ldg(chunkStart + chunk);
    c.n0 = __ldg(levelCnt + chunk * L);
    c.n1 = L > 1 ? __ldg(levelCnt + chunk * L + 1) : 0u;
#pragma unroll
    for (int i = 0; i < kRunsPerThread; i++) {
        const unsigned j = tid + kThreads * i;
        c.r0[i] = j < c.n0 ? __ldg(rec + c.start + j) : make_uint2(0xFFFFFFFFu, 0u);
    }
    c.r1 = tid < c.n1 ? __ldg(rec + c.start + c.n0 + tid) : make_uint2(0xFFFFFFFFu, 0u);
}

// One record into the running partial sum q: q + fl(gamma*T) * V[s'].
__device__ __forceinline__ float apply_record(float q, uint2 r, const float *vtile, unsigned tileLen) {
    const unsigned off = r.x & 0xFFFFu;
    return off < tileLen ? fadd(q, fmul(__uint_as_float(r.y), vtile[off])) : q;
}

// Run j of a chunk: its level-0 record r0, then (j < n1) the further
// levels in list order; first1 is the level-1 record when already loaded.
__device__ __forceinline__ void apply_run(uint2 r0, bool have1, uint2 first1, unsigned j, const ChunkRegs &c,
                                          const uint2 *__restrict__ rec, const unsigned *__restrict__ levelCnt,
                                          unsigned L, size_t chunk, const float *vtile, unsigned tileLen,
                                          float *part, unsigned rows) {
    const unsigned row = r0.x >> 16;
    if (row >= rows) return;
    float q = apply_record(part[row], r0, vtile, tileLen);
    if (j < c.n1) {
        q = apply_record(q, have1 ? first1 : __ldg(rec + c.start + c.n0 + j), vtile, tileLen);
        unsigned base = c.n0 + c.n1;
        for (unsigned lv = 2; lv < L; lv++) {
            const unsigned nq = __ldg(levelCnt + chunk * L + lv);
            if (j >= nq) break;
            q = apply_record(q, __ldg(rec + c.start + base + j), vtile, tileLen);
            base += nq;
        }
    }
    part[row] = q;
}

__global__ void __launch_bounds__(kThreads, 1) bellman_tiled_kernel(
        unsigned n, unsigned m, unsigned Vt, unsigned T, unsigned Sb, unsigned blocks, unsigned L,
        const uint2 *__restrict__ rec, const unsigned *__restrict__ chunkStart,
        const unsigned *__restrict__ levelCnt, const float *__restrict__ R, const float *__restrict__ V,
        float *__restrict__ Vp, unsigned *__restrict__ pi, ViDeviceState *st, double tol, int early_exit) {
    if (early_exit && *(volatile unsigned *)&st->converged) return;  // uniform across the grid
    extern __shared__ __align__(16) unsigned char smem[];
    float *vt = reinterpret_cast<float *>(smem);            // [2][Vt]
    float *part = vt + 2 * (size_t)Vt;                      // [Sb*m]
    const unsigned tid = threadIdx.x;
    double local = 0.0;
    for (unsigned blk = blockIdx.x; blk < blocks; blk += gridDim.x) {
        const unsigned s0 = blk * Sb;
        const unsigned nsb = min(Sb, n - s0);
        const unsigned rows = nsb * m;
        for (unsigned i = tid; i < rows; i += blockDim.x) part[i] = __ldg(R + (size_t)s0 * m + i);
        const size_t c0 = (size_t)blk * T;
        stage_tile(vt, V, n, 0, Vt);
        if (tid == 0) {
            prefetch_l2(rec, __ldg(chunkStart + c0), __ldg(chunkStart + c0 + min(T, 2u)));
        }
        ChunkRegs cur, nxt;
        load_chunk(cur, rec, chunkStart, levelCnt, L, c0, tid);
        cp_async_wait_all();
        __syncthreads();
        for (unsigned t = 0; t < T; t++) {
            const float *vcur = vt + (size_t)(t & 1) * Vt;
            const size_t chunk = c0 + t;
            if (t + 1 < T) {
                // The other buffer held tile t-1; every thread passed the
                // barrier that ended tile t-1, so it is free.
                stage_tile(vt + (size_t)((t + 1) & 1) * Vt, V, n, t + 1, Vt);
                if (tid == 0 && t + 2 < T)
                    prefetch_l2(rec, __ldg(chunkStart + chunk + 2), __ldg(chunkStart + chunk + 3));
                load_chunk(nxt, rec, chunkStart, levelCnt, L, chunk + 1, tid);
            }
            const unsigned tileLen = min(Vt, n - t * Vt);
#pragma unroll
            for (int i = 0; i < kRunsPerThread; i++) {
                const unsigned j = tid + kThreads * i;
                if (j < cur.n0)
                    apply_run(cur.r0[i], i == 0, cur.r1, j, cur, rec, levelCnt, L, chunk, vcur, tileLen, part,
                              rows);
            }
            for (unsigned j = tid + kThreads * kRunsPerThread; j < cur.n0; j += kThreads)
                apply_run(__ldg(rec + cur.start + j), false, cur.r1, j, cur, rec, levelCnt, L, chunk, vcur, tileLen,
                          part, rows);
            cp_async_wait_all();
            __syncthreads();
            cur = nxt;
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
    unsigned n, m, ns, Vt, T, Sb, L;
    float gamma;
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

__device__ __forceinline__ unsigned run_cell(unsigned rowLocal, unsigned off) {
    const unsigned qb = rowLocal & 31u, vb = off & 31u;
    return qb * 32u + ((vb - qb) & 31u);
}

// Per chunk c = block * T + tile: levelCnt[c*L + q] = runs with more than q
// records; cell[c*1024 + qb*32 + d] = single-record runs whose partial sum
// is in bank qb at distance d; longCnt[c*(L+1) + len] = runs of len >= 2.
__global__ void vi_plan_count_kernel(PlanGeometry g, const int *__restrict__ S, unsigned *__restrict__ levelCnt,
                                     unsigned *__restrict__ cell, unsigned *__restrict__ longCnt) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)g.n * g.m) return;
    const unsigned blk = (unsigned)(row / g.m) / g.Sb;
    const unsigned rowLocal = (unsigned)(row - (unsigned long long)blk * g.Sb * g.m);
    const int *Sr = S + row * g.ns;
    for_each_run(Sr, g.ns, g.Vt, [&](unsigned t, unsigned l0, unsigned len) {
        const size_t c = (size_t)blk * g.T + t;
        for (unsigned q = 0; q < len; q++) atomicAdd(levelCnt + c * g.L + q, 1u);
        if (len == 1) atomicAdd(cell + c * 1024 + run_cell(rowLocal, (unsigned)Sr[l0] - t * g.Vt), 1u);
        else atomicAdd(longCnt + c * (g.L + 1) + len, 1u);
    });
}

// Per chunk: its record count; each partial-sum bank's bucket size (bsize)
// and, in place, the bucket's exclusive prefix over distances (cell); the
// long runs' exclusive prefix by length, longest first (longCnt).
__global__ void vi_plan_chunk_kernel(unsigned nChunks, unsigned L, const unsigned *__restrict__ levelCnt,
                                     unsigned *__restrict__ cell, unsigned *__restrict__ bsize,
                                     unsigned *__restrict__ longCnt, unsigned *__restrict__ chunkSize) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nChunks) return;
    unsigned total = 0;
    for (unsigned q = 0; q < L; q++) total += levelCnt[c * L + q];
    chunkSize[c] = total;
    for (unsigned qb = 0; qb < 32; qb++) {
        unsigned *b = cell + c * 1024 + qb * 32;
        unsigned run = 0;
        for (unsigned d = 0; d < 32; d++) {
            const unsigned v = b[d];
            b[d] = run;
            run += v;
        }
        bsize[c * 32 + qb] = run;
    }
    unsigned run = 0;
    for (unsigned len = L; len >= 2; len--) {
        unsigned *p = longCnt + c * (L + 1) + len;
        const unsigned v = *p;
        *p = run;
        run += v;
    }
}

// Write every record at its place. The position j of a run in its chunk's
// levels: long runs first, by length (ties in the order threads arrive,
// which changes nothing: the rows of one chunk are distinct), then the
// single-record runs dealt round-robin over the 32 partial-sum banks, the
// k-th run of a bank's bucket (sorted by distance) in round k.
__global__ void vi_plan_fill_kernel(PlanGeometry g, const int *__restrict__ S, const float *__restrict__ Tm,
                                    const unsigned *__restrict__ chunkStart, const unsigned *__restrict__ levelCnt,
                                    unsigned *__restrict__ cell, const unsigned *__restrict__ bsize,
                                    unsigned *__restrict__ longCnt, uint2 *__restrict__ rec) {
    const unsigned long long row = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= (unsigned long long)g.n * g.m) return;
    const unsigned blk = (unsigned)(row / g.m) / g.Sb;
    const unsigned rowLocal = (unsigned)(row - (unsigned long long)blk * g.Sb * g.m);
    const int *Sr = S + row * g.ns;
    const float *Tr = Tm + row * g.ns;
    for_each_run(Sr, g.ns, g.Vt, [&](unsigned t, unsigned l0, unsigned len) {
        const size_t c = (size_t)blk * g.T + t;
        unsigned j;
        if (len >= 2) {
            j = atomicAdd(longCnt + c * (g.L + 1) + len, 1u);
        } else {
            const unsigned ce = run_cell(rowLocal, (unsigned)Sr[l0] - t * g.Vt);
            const unsigned qb = ce >> 5;
            const unsigned rank = atomicAdd(cell + c * 1024 + ce, 1u);
            j = g.L > 1 ? levelCnt[c * g.L + 1] : 0u;   // the long runs come first
            const unsigned *bs = bsize + c * 32;
            for (unsigned b = 0; b < 32; b++) {
                const unsigned sz = bs[b];
                j += min(sz, rank) + ((b < qb && sz > rank) ? 1u : 0u);
            }
        }
        unsigned base = chunkStart[c];
        for (unsigned q = 0; q < len; q++) {
            const unsigned sp = (unsigned)Sr[l0 + q];
            rec[base + j] = make_uint2((rowLocal << 16) | (sp - t * g.Vt), __float_as_uint(fmul(g.gamma, Tr[l0 + q])));
            base += levelCnt[c * g.L + q];
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
    cudaFree(plan->chunkStart);
    cudaFree(plan->levelCnt);
    cudaFree(plan->flags);
    plan->rec = nullptr;
    plan->chunkStart = plan->levelCnt = plan->flags = nullptr;
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
    if (hflags[0] != 0 || hflags[1] != 0 || L > kMaxLevels) {
        release(plan);
        return NOVA_SUCCESS;
    }
    const PlanGeometry g{n, m, ns, Vt, tiles, Sb, L, mdp->gamma};
    const unsigned long long nChunks = (unsigned long long)blocks * tiles;
    if (nChunks * 1024ull >= (1ull << 32) || nChunks * (L + 1) >= (1ull << 32)) { release(plan); return NOVA_SUCCESS; }

    // Pass 2: per-chunk counts (levels, bank cells, long runs).
    unsigned *cell = nullptr, *bsize = nullptr, *longCnt = nullptr, *chunkSize = nullptr;
    auto freeScratch = [&]() {
        cudaFree(cell); cudaFree(bsize); cudaFree(longCnt); cudaFree(chunkSize);
        cell = bsize = longCnt = chunkSize = nullptr;
    };
    if (!try_alloc(&plan->levelCnt, nChunks * L) || !try_alloc(&cell, nChunks * 1024) ||
            !try_alloc(&bsize, nChunks * 32) || !try_alloc(&longCnt, nChunks * (L + 1)) ||
            !try_alloc(&chunkSize, nChunks) || !try_alloc(&plan->chunkStart, nChunks + 1)) {
        freeScratch();
        release(plan);
        return NOVA_SUCCESS;
    }
    if (cudaMemsetAsync(plan->levelCnt, 0, nChunks * L * sizeof(unsigned), stream) != cudaSuccess ||
            cudaMemsetAsync(cell, 0, nChunks * 1024 * sizeof(unsigned), stream) != cudaSuccess ||
            cudaMemsetAsync(longCnt, 0, nChunks * (L + 1) * sizeof(unsigned), stream) != cudaSuccess) {
        cudaGetLastError();
        freeScratch();
        release(plan);
        NOVA_ERR(fn, "Failed to clear the sweep plan counters.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    vi_plan_count_kernel<<<rowBlocks, 256, 0, stream>>>(g, S, plan->levelCnt, cell, longCnt);
    rc = check_launch(fn, "sweep plan (count)");
    if (rc == NOVA_SUCCESS) {
        vi_plan_chunk_kernel<<<ceil_div(nChunks, 128), 128, 0, stream>>>((unsigned)nChunks, L, plan->levelCnt, cell,
                                                                         bsize, longCnt, chunkSize);
        rc = check_launch(fn, "sweep plan (chunks)");
    }
    if (rc == NOVA_SUCCESS) rc = scan_counts(chunkSize, nChunks, plan->chunkStart, stream, fn);
    unsigned total = 0;
    if (rc == NOVA_SUCCESS)
        rc = d2h(&total, plan->chunkStart + nChunks, sizeof(unsigned), fn, "the sweep plan size");
    // Pass 3: the records (two spare ones at the end for the bulk prefetch).
    if (rc == NOVA_SUCCESS && !try_alloc(&plan->rec, (size_t)total + 2)) rc = NOVA_ERROR_DEVICE_MALLOC;
    if (rc == NOVA_SUCCESS &&
            cudaMemsetAsync(plan->rec, 0xFF, ((size_t)total + 2) * sizeof(uint2), stream) != cudaSuccess) {
        cudaGetLastError();
        rc = NOVA_ERROR_KERNEL_EXECUTION;
    }
    if (rc == NOVA_SUCCESS) {
        vi_plan_fill_kernel<<<rowBlocks, 256, 0, stream>>>(g, S, T, plan->chunkStart, plan->levelCnt, cell, bsize,
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
        plan->chunkStart, plan->levelCnt, R, V, Vp, pi, st, tol, early_exit);
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
