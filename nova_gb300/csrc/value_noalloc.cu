// nova-gb300: V(b) of a device-resident alpha-vector policy without any
// device allocation.
//
// Some callers must not call cudaMalloc while they run: a controller that
// evaluates its policy at every belief inside a real-time loop (an
// allocation can block on device-wide synchronisation and take
// unpredictable time), or a process whose device memory is owned by another
// framework's pool. pomdp_pbvi_value_gpu needs a solver workspace for its
// per-alpha FP64 values; this variant keeps that scratch in a fixed
// file-scope device array instead, so a call only launches kernels and
// copies the 12-byte result back.
//
// The scratch holds NOVA_VALUE_NOALLOC_MAX_ROWS doubles plus the result, and
// every GPU that loads this library keeps it until the process exits. All
// calls share it: two calls whose kernels overlap on the GPU (different
// host threads, or different streams of the caller) race on it, so callers
// must serialise them. The first call on a device (and the first call after
// the device's context was created anew, e.g. after cudaDeviceReset)
// resolves the array's device address for that device
// (cudaGetSymbolAddress); make that first call before any stream capture.
// Kernels run on the calling thread's per-thread default stream (the library
// is built with per-thread default streams): work that writes d_Gamma, d_pi
// or d_b on other streams or host threads must be complete before the call.

#include "common.h"

#include <nova/constants.h>
#include <nova/nova_gb300.h>

namespace nova_gb300 {

constexpr unsigned kNoAllocMaxRows = NOVA_VALUE_NOALLOC_MAX_ROWS;
constexpr unsigned kNoneN = 0xffffffffu;

struct NoAllocScratch {
    double rowValue[kNoAllocMaxRows];  // b . Gamma_i in FP64, one per alpha
    double bestValue;                  // result: V(b)
    unsigned bestAction;               // result: pi of the maximising alpha
    unsigned pad;
};

// The scratch. In host code this name is a host-side stand-in, not a device
// address: host code only ever passes the address that cudaGetSymbolAddress
// returns for the current device.
static __device__ __align__(256) NoAllocScratch g_value_scratch;

__global__ void noalloc_row_value_kernel(const float *__restrict__ G, unsigned n, const float *__restrict__ b,
                                         NoAllocScratch *scratch) {
    const unsigned j = blockIdx.x;
    double acc = 0.0;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) acc += (double)G[(size_t)j * n + s] * (double)b[s];
    __shared__ double red[32];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned w = 0; w < (blockDim.x + 31) / 32; w++) t += red[w];
        scratch->rowValue[j] = t;
    }
}

// Maximum with the lowest index on ties and the -1e10 start of
// pomdp_alpha_vectors.cpp:52-79; writes both result fields every call.
__global__ void noalloc_argmax_kernel(unsigned rows, const unsigned *__restrict__ pi, NoAllocScratch *scratch) {
    double best = (double)NOVA_FLT_MIN;
    unsigned bi = kNoneN;
    for (unsigned j = threadIdx.x; j < rows; j += blockDim.x) {
        const double v = scratch->rowValue[j];
        if (v > best) { best = v; bi = j; }
    }
    __shared__ double sv[256];
    __shared__ unsigned si[256];
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (unsigned t = 1; t < blockDim.x; t++) {
            if (si[t] == kNoneN) continue;
            if (si[0] == kNoneN || sv[t] > sv[0] || (sv[t] == sv[0] && si[t] < si[0])) { sv[0] = sv[t]; si[0] = si[t]; }
        }
        scratch->bestValue = sv[0];
        scratch->bestAction = si[0] == kNoneN ? 0u : pi[si[0]];
    }
}

// Device address of the scratch, resolved once per device and context. A
// context created anew on a device (after cudaDeviceReset, or when the
// primary context was released and retained again) loads this module again
// at a new address, so the cached address is kept together with the context
// it belongs to and resolved again when the current context differs.
typedef int (*CtxGetCurrentFn)(void **);

static CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn f = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    return f;
}

static std::mutex g_scratch_mutex;
static NoAllocScratch *g_scratch_addr[64] = {};
static void *g_scratch_ctx[64] = {};

static int scratch_for_current_device(NoAllocScratch **out, const char *fn) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        NOVA_ERR(fn, "No usable current CUDA device.");
        return NOVA_ERROR_INVALID_CUDA_PARAM;
    }
    // cudaGetSymbolAddress makes the device's primary context current when
    // no context is, so the context is read after it on the first call.
    void *ctx = nullptr;
    CtxGetCurrentFn getCtx = ctx_get_current();
    if (getCtx != nullptr && getCtx(&ctx) != 0) ctx = nullptr;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_addr[dev] == nullptr || ctx == nullptr || ctx != g_scratch_ctx[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_value_scratch) != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            NOVA_ERR(fn, "Failed to resolve the device address of the evaluation scratch.");
            return NOVA_ERROR_KERNEL_EXECUTION;
        }
        if (getCtx != nullptr && getCtx(&ctx) != 0) ctx = nullptr;
        g_scratch_addr[dev] = static_cast<NoAllocScratch *>(p);
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_addr[dev];
    return NOVA_SUCCESS;
}

}  // namespace nova_gb300

using namespace nova_gb300;

extern "C" int pomdp_alpha_vectors_value_noalloc_gpu(const float *d_Gamma, const unsigned int *d_pi, unsigned int r,
                                                     unsigned int n, const float *d_b, double *Vb, unsigned int *a) {
    static const char *fn = "pomdp_alpha_vectors_value_noalloc_gpu";
    if (d_Gamma == nullptr || d_pi == nullptr || d_b == nullptr || Vb == nullptr || a == nullptr || r == 0 || n == 0) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (r > kNoAllocMaxRows) {
        NOVA_ERR(fn, "Too many alpha-vectors: the allocation-free evaluation holds at most "
                     "NOVA_VALUE_NOALLOC_MAX_ROWS (65536) of them; use pomdp_pbvi_value_gpu.");
        return NOVA_ERROR_INVALID_DATA;
    }
    NoAllocScratch *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch, fn);
    if (rc != NOVA_SUCCESS) return rc;
    // Every field the argmax reads is written by the row kernel of this call,
    // and both result fields are written by the argmax kernel, so nothing
    // left by an earlier call is read.
    noalloc_row_value_kernel<<<r, 256>>>(d_Gamma, n, d_b, scratch);
    if ((rc = check_launch(fn, "FP64 belief values")) != NOVA_SUCCESS) return rc;
    noalloc_argmax_kernel<<<1, 256>>>(r, d_pi, scratch);
    if ((rc = check_launch(fn, "FP64 belief argmax")) != NOVA_SUCCESS) return rc;
    double v = 0.0;
    unsigned act = 0;
    if ((rc = d2h(&v, &scratch->bestValue, sizeof(double), fn, "the value")) != NOVA_SUCCESS) return rc;
    if ((rc = d2h(&act, &scratch->bestAction, sizeof(unsigned), fn, "the action")) != NOVA_SUCCESS) return rc;
    *Vb = v;
    *a = act;
    return NOVA_SUCCESS;
}
