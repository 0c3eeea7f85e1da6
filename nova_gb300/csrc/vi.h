// nova-gb300 internal header: state shared by the two Bellman sweep kernels
// (the per-row gather sweep in mdp_vi.cu and the column-tiled sweep in
// mdp_vi_tiled.cu).
#pragma once

#include "common.h"

#include <nova/mdp/mdp.h>

namespace nova_gb300 {

// Convergence bookkeeping shared by the sweep kernels of one solver.
struct ViDeviceState {
    unsigned long long resid_bits;   // max |V' - V| of the current sweep, as FP64 bits
    unsigned int blocks_done;        // blocks finished in the current sweep
    unsigned int sweeps_done;        // sweeps that ran (early-exit mode)
    unsigned int converged;          // 1 once a sweep's residual fell below tol
    unsigned int err;                // 1 if a bounded wait of the tiled sweep ran out
    double last_resid;               // residual of the last finished sweep
};

#ifdef __CUDACC__
__device__ __forceinline__ void residual_commit(double local, ViDeviceState *st, unsigned nblocks, double tol,
                                                bool early_exit) {
    // Block max, then one FP64 atomic max (non-negative doubles order like
    // their bit patterns), then the last block closes the sweep.
    __shared__ double red[32];
    for (int off = 16; off > 0; off >>= 1) local = fmax(local, __shfl_xor_sync(0xffffffffu, local, off));
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[warp] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (unsigned w = 0; w < (blockDim.x + 31) / 32; w++) m = fmax(m, red[w]);
        atomicMax(&st->resid_bits, (unsigned long long)__double_as_longlong(m));
        __threadfence();
        const unsigned done = atomicAdd(&st->blocks_done, 1u);
        if (done == nblocks - 1) {
            __threadfence();
            const double r = __longlong_as_double((long long)atomicAdd(&st->resid_bits, 0ull));
            st->last_resid = r;
            st->resid_bits = 0ull;
            st->blocks_done = 0u;
            st->sweeps_done += 1u;
            if (early_exit && r < tol) st->converged = 1u;
            __threadfence();
        }
    }
}
#endif

// Tile plan of the column-tiled sweep: the model's successor entries
// regrouped by slice (block of source states, tile of successor states, row
// warp) and, within a slice, by level, where level q holds the q-th
// successor of each row inside the tile. Built once per solver from the
// device copies of S and T.
struct ViTilePlan {
    enum Status : unsigned { kNotBuilt = 0, kTiled = 1, kGather = 2 };
    Status status = kNotBuilt;
    unsigned tileStates = 0;    // states per shared-memory tile of V (multiple of 4)
    unsigned tiles = 0;         // ceil(n / tileStates)
    unsigned blockStates = 0;   // source states per block
    unsigned blocks = 0;        // ceil(n / blockStates)
    unsigned levels = 0;        // longest run of one row's successors inside one tile
    unsigned grid = 0;          // resident CTAs
    size_t smemBytes = 0;
    uint2 *rec = nullptr;          // [entries + 2] {row << 16 | byte offset in tile, bits of fl(gamma * T)}
    unsigned *sliceStart = nullptr;  // [blocks*tiles*rowWarps + 1] first record of each (block, tile, warp) slice
    uint4 *sliceHdr = nullptr;       // [slices + pad] {first record, runs, runs with 2+ records, runs with 3+}
    unsigned *levelCnt = nullptr;    // [slices][levels] runs of each slice with more than q records
    unsigned *flags = nullptr;     // build scratch: unsorted rows, out-of-range successor, longest run
    ~ViTilePlan();
};

// Build the plan for the model (dimensions from mdp, arrays S and T on the
// device) unless it is built already. Leaves status kTiled or kGather; a
// failed device allocation leaves kGather. Returns a NOVA_* code only for
// launch or copy errors.
int vi_plan_build(ViTilePlan *plan, const nova::MDP *mdp, const int *S, const float *T, cudaStream_t stream,
                  const char *fn);

// One tiled sweep V -> Vp (plan status kTiled, V 16-byte aligned).
int vi_tiled_sweep(const ViTilePlan *plan, const nova::MDP *mdp, const float *R, const float *V, float *Vp,
                   unsigned *pi, ViDeviceState *st, double tol, int early_exit, cudaStream_t stream,
                   const char *fn);

// Reads (and clears) the state's error word after the sweeps queued so far
// finished: NOVA_ERROR_KERNEL_EXECUTION if a bounded wait ran out.
int vi_state_error(ViDeviceState *st, const char *fn);

// Status of the plan built last in this process (ViTilePlan::Status).
unsigned vi_last_plan_status();

}  // namespace nova_gb300
