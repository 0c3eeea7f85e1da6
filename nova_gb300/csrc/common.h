// nova-gb300 internal header: CUDA wrappers with NOVA_* error mapping,
// host-side fault injection, the per-solver workspace registry and small
// device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <memory>

#include <nova/error_codes.h>

namespace nova_gb300 {

// ---------------------------------------------------------------------------
// Error reporting. Messages follow the reference's "Error[<fn>]: <msg>" form
// (e.g. pomdp_pbvi_gpu.cu:219-228) on stderr.
// ---------------------------------------------------------------------------
#define NOVA_ERR(fn, msg) fprintf(stderr, "Error[%s]: %s\n", fn, msg)

// Fault injection: the count-th call of a wrapper of the armed kind fails.
enum FaultKind : unsigned { kFaultNone = 0, kFaultMalloc = 1, kFaultH2D = 2, kFaultD2H = 3, kFaultLaunch = 4 };
bool fault_fires(FaultKind kind);

int dev_malloc(void **p, size_t bytes, const char *fn, const char *what);
int dev_free(void *p, const char *fn, const char *what);
int h2d(void *dst, const void *src, size_t bytes, const char *fn, const char *what);
int d2h(void *dst, const void *src, size_t bytes, const char *fn, const char *what);
int check_launch(const char *fn, const char *what);  // call once after every kernel launch
unsigned long long launch_count();
void add_launches(long long delta);  // kernels run by a graph replay (negative: captured, not run)
int sync_device(const char *fn);

template <typename T>
inline int dev_alloc(T **p, size_t count, const char *fn, const char *what) {
    return dev_malloc(reinterpret_cast<void **>(p), count * sizeof(T), fn, what);
}

// Device-side error word: bounded waits write a code here instead of hanging.
// Codes: 1 = mbarrier wait timed out in the scoring GEMM. Defined with the
// kernels that wait (pbvi_tc.cu).
unsigned read_and_clear_device_error();

// ---------------------------------------------------------------------------
// Per-solver workspace registry keyed by the address of the caller's solver
// struct (POMDPPBVIGPU, MDPVIGPU, ...). It lets initialize be idempotent and
// keeps workspace that the reference structs have no field for.
// ---------------------------------------------------------------------------
struct Workspace {
    virtual ~Workspace() = default;
};

std::mutex &registry_mutex();
std::unordered_map<const void *, std::unique_ptr<Workspace>> &registry();

template <typename W>
W *find_workspace(const void *key) {
    auto &reg = registry();
    auto it = reg.find(key);
    if (it == reg.end()) return nullptr;
    return dynamic_cast<W *>(it->second.get());
}

// Bounded spin budget for device-side waits (iterations of try_wait).
constexpr unsigned long long kWaitLimit = 1ull << 26;

inline unsigned ceil_div(unsigned long long a, unsigned long long b) {
    return (unsigned)((a + b - 1) / b);
}
inline size_t round_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

}  // namespace nova_gb300

#ifdef __CUDACC__
namespace nova_gb300 {
// IEEE single-precision add/multiply with round-to-nearest and no
// contraction into FMA: the reference's CPU path (g++ without FMA) rounds
// every product and every sum, and matching those bits requires the same.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }

// Packed pairs of FP32 values (element 0 in the low word): the sm_100-family
// f32x2 multiply rounds each element exactly as the scalar multiply. For the
// sum use fma_f32x2(p, one, acc) with one = 1.0 passed in at run time: p * 1
// is exact, so the result is the correctly rounded acc + p, whereas an
// add.rn.f32x2 that consumes an f32x2 product is contracted by the compiler
// into one fused multiply-add (the product's rounding skipped).
__device__ __forceinline__ unsigned long long pack_f32x2(float lo, float hi) {
    unsigned long long d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ unsigned long long mul_f32x2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long fma_f32x2(unsigned long long a, unsigned long long b,
                                                       unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ float f32x2_part(unsigned long long v, int hi) {
    return __uint_as_float(hi ? (unsigned)(v >> 32) : (unsigned)v);
}
}  // namespace nova_gb300
#endif
