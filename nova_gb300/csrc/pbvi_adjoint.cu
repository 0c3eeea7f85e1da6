// nova-gb300: reverse mode of H recorded PBVI backups.
//
// With the selections of every backup held fixed (for belief i at step t:
// the action a whose alpha became Gamma_t[i], and per observation o the
// alpha index j_o chosen for (i, a, o)), a backup is the smooth map
//
//   Gamma_t[i](s) = R(s,a) + sum_o gamma * sum_l O(a,S(s,a,l),o) T(s,a,l) Gamma_{t-1}[j_o](S(s,a,l))
//
// (pomdp_pbvi_cpu.cpp:37-103 with its argmax results recorded), and
// V(b0) = b0 . Gamma_H[i*] with i* = argmax_i b0 . Gamma_H[i]
// (pomdp_alpha_vectors.cpp:52-79). This file differentiates V(b0) with
// respect to R, T and O (and Gamma_0) by the adjoint recursion, for
// lambda_t = dV/dGamma_t (r x n, FP64):
//
//   dR(s,a)          += lambda_t[i](s)
//   c_i(s')           = sum_o O(a,s',o) Gamma_{t-1}[j_o](s')
//   dT(s,a,l)        += gamma * lambda_t[i](s) * c_i(S(s,a,l))
//   w_i(s')           = sum_{(s,l): S(s,a,l)=s'} T(s,a,l) lambda_t[i](s)
//   dO(a,s',o)       += gamma * w_i(s') * Gamma_{t-1}[j_o](s')
//   lambda_{t-1}[j_o](s') += gamma * O(a,s',o) * w_i(s')
//
// Gamma_{t-1} is needed at every reverse step. The caller keeps
// checkpoints every k steps; each segment between checkpoints is
// recomputed forward in FP32 with the recorded selections, in the
// reference's operation order, so the recomputed alphas are bit-identical
// to the forward pass.

#include "common.h"

#include <algorithm>
#include <vector>

#include <nova/constants.h>
#include <nova/pomdp/pomdp.h>
#include <nova/pomdp/algorithms/pomdp_pbvi_gpu.h>
#include <nova/nova_gb300.h>

using nova::POMDP;
using nova::POMDPPBVIGPU;

namespace nova_gb300 {
namespace {

constexpr unsigned kNoRow = 0xffffffffu;

struct AdjModel {
    unsigned n, ns, m, z, r;
    float gamma;
    const int *S;
    const float *T, *O, *R;
};

__global__ void adj_len_kernel(unsigned rows, unsigned ns, const int *__restrict__ S, unsigned *__restrict__ len) {
    const unsigned row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    unsigned L = ns;
    for (unsigned l = 0; l < ns; l++)
        if (S[(size_t)row * ns + l] < 0) { L = l; break; }
    len[row] = L;
}

// C3[a][o][s][l] = fl(O(a,S(s,a,l),o) * T(s,a,l)) (the reference's first
// product), 0 past the row end.
__global__ void adj_coef_kernel(AdjModel md, const unsigned *__restrict__ len, float *__restrict__ C3) {
    const size_t total = (size_t)md.m * md.z * md.n * md.ns;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const unsigned l = (unsigned)(e % md.ns);
        size_t t = e / md.ns;
        const unsigned s = (unsigned)(t % md.n);
        t /= md.n;
        const unsigned o = (unsigned)(t % md.z);
        const unsigned a = (unsigned)(t / md.z);
        float c = 0.0f;
        if (l < len[(size_t)s * md.m + a]) {
            const size_t row = ((size_t)s * md.m + a) * md.ns + l;
            c = fmul(md.O[((size_t)a * md.n + md.S[row]) * md.z + o], md.T[row]);
        }
        C3[e] = c;
    }
}

// Gamma_t from Gamma_{t-1} with recorded selections, in the reference's
// order: alpha = R(s,a); for each o, alpha += gamma * sum_l C3 * G_j(S).
__global__ void replay_kernel(AdjModel md, const unsigned *__restrict__ len, const float *__restrict__ C3,
                              const float *__restrict__ Gin, const unsigned *__restrict__ act,
                              const unsigned *__restrict__ sel, float *__restrict__ Gout) {
    const unsigned i = blockIdx.x;
    extern __shared__ unsigned jsh[];  // [z]
    const unsigned a = min(act[i], md.m - 1);
    for (unsigned o = threadIdx.x; o < md.z; o += blockDim.x) jsh[o] = min(sel[(size_t)i * md.z + o], md.r - 1);
    __syncthreads();
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        float alpha = md.R[(size_t)s * md.m + a];
        const unsigned L = len[(size_t)s * md.m + a];
        const int *sp = md.S + ((size_t)s * md.m + a) * md.ns;
        for (unsigned o = 0; o < md.z; o++) {
            const float *c = C3 + (((size_t)a * md.z + o) * md.n + s) * md.ns;
            const float *Gj = Gin + (size_t)jsh[o] * md.n;
            float vt = 0.0f;
            for (unsigned l = 0; l < L; l++) vt = fadd(vt, fmul(c[l], Gj[sp[l]]));
            alpha = fadd(alpha, fmul(vt, md.gamma));
        }
        Gout[(size_t)i * md.n + s] = alpha;
    }
}

// vals[i] = b . Gamma[i] in FP64.
__global__ void value_rows_kernel(const float *__restrict__ G, unsigned n, const float *__restrict__ b,
                                  double *__restrict__ vals) {
    const unsigned i = blockIdx.x;
    double acc = 0.0;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) acc += (double)G[(size_t)i * n + s] * (double)b[s];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned w = 0; w < blockDim.x / 32; w++) t += red[w];
        vals[i] = t;
    }
}

// Maximum with the -1e10 start and lowest index on ties; seeds
// lambda_H[i*] = b.
__global__ void value_argmax_kernel(unsigned r, unsigned n, const double *__restrict__ vals,
                                    const float *__restrict__ b, double *__restrict__ Vout,
                                    unsigned *__restrict__ iout, double *__restrict__ lam) {
    __shared__ double sv[256];
    __shared__ unsigned si[256];
    double best = (double)NOVA_FLT_MIN;
    unsigned bi = kNoRow;
    for (unsigned j = threadIdx.x; j < r; j += blockDim.x)
        if (vals[j] > best) { best = vals[j]; bi = j; }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    __shared__ unsigned istar;
    if (threadIdx.x == 0) {
        for (unsigned t = 1; t < blockDim.x; t++) {
            if (si[t] == kNoRow) continue;
            if (si[0] == kNoRow || sv[t] > sv[0] || (sv[t] == sv[0] && si[t] < si[0])) { sv[0] = sv[t]; si[0] = si[t]; }
        }
        *Vout = sv[0];
        *iout = si[0];
        istar = si[0];
    }
    __syncthreads();
    if (istar == kNoRow) return;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) lam[(size_t)istar * n + s] = (double)b[s];
}

// One reverse step for belief i = blockIdx.x. Shared memory: c_i and w_i
// (n doubles each) and the z selections.
__global__ void adjoint_step_kernel(AdjModel md, const unsigned *__restrict__ len, const float *__restrict__ Gprev,
                                    const unsigned *__restrict__ act, const unsigned *__restrict__ sel,
                                    const double *__restrict__ lam, double *__restrict__ lamPrev,
                                    double *__restrict__ dR, double *__restrict__ dT, double *__restrict__ dO) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *csh = reinterpret_cast<double *>(smem);
    double *wsh = csh + md.n;
    unsigned *jsh = reinterpret_cast<unsigned *>(wsh + md.n);
    const unsigned i = blockIdx.x;
    const double *lrow = lam + (size_t)i * md.n;
    bool nz = false;
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) nz |= lrow[s] != 0.0;
    if (!__syncthreads_or(nz)) return;
    const unsigned a = min(act[i], md.m - 1);
    for (unsigned o = threadIdx.x; o < md.z; o += blockDim.x) jsh[o] = min(sel[(size_t)i * md.z + o], md.r - 1);
    __syncthreads();
    const double g = (double)md.gamma;
    for (unsigned sp = threadIdx.x; sp < md.n; sp += blockDim.x) {
        const float *Orow = md.O + ((size_t)a * md.n + sp) * md.z;
        double c = 0.0;
        for (unsigned o = 0; o < md.z; o++) c += (double)Orow[o] * (double)Gprev[(size_t)jsh[o] * md.n + sp];
        csh[sp] = c;
        wsh[sp] = 0.0;
    }
    __syncthreads();
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        const double l = lrow[s];
        if (l == 0.0) continue;
        atomicAdd(dR + (size_t)s * md.m + a, l);
        const size_t row = ((size_t)s * md.m + a) * md.ns;
        const unsigned L = len[(size_t)s * md.m + a];
        for (unsigned k = 0; k < L; k++) {
            const unsigned sp = (unsigned)md.S[row + k];
            atomicAdd(wsh + sp, (double)md.T[row + k] * l);
            atomicAdd(dT + row + k, g * l * csh[sp]);
        }
    }
    __syncthreads();
    for (unsigned sp = threadIdx.x; sp < md.n; sp += blockDim.x) {
        const double w = wsh[sp];
        if (w == 0.0) continue;
        const size_t ob = ((size_t)a * md.n + sp) * md.z;
        for (unsigned o = 0; o < md.z; o++) {
            const size_t gj = (size_t)jsh[o] * md.n + sp;
            atomicAdd(dO + ob + o, g * w * (double)Gprev[gj]);
            atomicAdd(lamPrev + gj, g * (double)md.O[ob + o] * w);
        }
    }
}

struct AdjBuffers {
    unsigned *len = nullptr;
    float *C3 = nullptr, *seg = nullptr;
    double *lamA = nullptr, *lamB = nullptr, *vals = nullptr, *V = nullptr;
    unsigned *istar = nullptr;
    ~AdjBuffers() {
        cudaFree(len); cudaFree(C3); cudaFree(seg);
        cudaFree(lamA); cudaFree(lamB); cudaFree(vals); cudaFree(V); cudaFree(istar);
    }
};

// Gamma_t from Gamma_{t-1} in FP64 with recorded selections:
// alpha(s) = R(s,a) + gamma * sum_l T(s,a,l) sum_o O(a,S,o) Gamma_{j_o}(S),
// every operand widened to FP64 (the same map as replay_kernel without the
// FP32 roundings; the order of the FP64 sums differs from the reference's).
__global__ void replay_f64_kernel(AdjModel md, const unsigned *__restrict__ len, const double *__restrict__ Gin,
                                  const unsigned *__restrict__ act, const unsigned *__restrict__ sel,
                                  double *__restrict__ Gout) {
    const unsigned i = blockIdx.x;
    extern __shared__ unsigned jsh[];  // [z]
    const unsigned a = min(act[i], md.m - 1);
    for (unsigned o = threadIdx.x; o < md.z; o += blockDim.x) jsh[o] = min(sel[(size_t)i * md.z + o], md.r - 1);
    __syncthreads();
    const double gamma = (double)md.gamma;
    for (unsigned s = threadIdx.x; s < md.n; s += blockDim.x) {
        const size_t row = (size_t)s * md.m + a;
        const unsigned L = len[row];
        double acc = 0.0;
        for (unsigned l = 0; l < L; l++) {
            const unsigned sp = (unsigned)md.S[row * md.ns + l];
            const float *Orow = md.O + ((size_t)a * md.n + sp) * md.z;
            double w = 0.0;
            for (unsigned o = 0; o < md.z; o++) w += (double)Orow[o] * Gin[(size_t)jsh[o] * md.n + sp];
            acc += (double)md.T[row * md.ns + l] * w;
        }
        Gout[(size_t)i * md.n + s] = (double)md.R[row] + gamma * acc;
    }
}

__global__ void widen_kernel(const float *__restrict__ in, size_t count, double *__restrict__ out) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (double)in[e];
}

// vals[i] = b . Gamma[i] with FP64 alphas.
__global__ void value_rows_f64_kernel(const double *__restrict__ G, unsigned n, const float *__restrict__ b,
                                      double *__restrict__ vals) {
    const unsigned i = blockIdx.x;
    double acc = 0.0;
    for (unsigned s = threadIdx.x; s < n; s += blockDim.x) acc += G[(size_t)i * n + s] * (double)b[s];
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    __shared__ double red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned w = 0; w < blockDim.x / 32; w++) t += red[w];
        vals[i] = t;
    }
}

}  // namespace
}  // namespace nova_gb300

using namespace nova_gb300;

extern "C" int pomdp_pbvi_adjoint_gpu(const POMDP *pomdp, unsigned int horizon, unsigned int checkpointEvery,
                                      const float *d_checkpoints, const unsigned int *d_actions,
                                      const unsigned int *d_selects, const float *d_b, double *d_dR, double *d_dT,
                                      double *d_dO, double *d_dGamma0, double *Vb, unsigned int *bestAlpha) {
    static const char *fn = "pomdp_pbvi_adjoint_gpu";
    if (pomdp == nullptr || pomdp->n == 0 || pomdp->ns == 0 || pomdp->m == 0 || pomdp->z == 0 || pomdp->r == 0 ||
            pomdp->d_S == nullptr || pomdp->d_T == nullptr || pomdp->d_O == nullptr || pomdp->d_R == nullptr ||
            horizon == 0 || checkpointEvery == 0 || d_checkpoints == nullptr || d_actions == nullptr ||
            d_selects == nullptr || d_b == nullptr || d_dR == nullptr || d_dT == nullptr || d_dO == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    AdjModel md{pomdp->n, pomdp->ns, pomdp->m, pomdp->z, pomdp->r, pomdp->gamma,
                pomdp->d_S, pomdp->d_T, pomdp->d_O, pomdp->d_R};
    const size_t stepSmem = 2 * (size_t)md.n * sizeof(double) + (size_t)md.z * sizeof(unsigned);
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
            stepSmem > (size_t)optin) {
        cudaGetLastError();
        NOVA_ERR(fn, "Too many states for the reverse step's shared-memory buffers.");
        return NOVA_ERROR_INVALID_DATA;
    }
    if (stepSmem > 48 * 1024 &&
            cudaFuncSetAttribute(adjoint_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stepSmem) !=
                cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to configure the reverse step kernel.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    const unsigned n = md.n, r = md.r, z = md.z, m = md.m, ns = md.ns, k = checkpointEvery;
    const size_t rn = (size_t)r * n;
    AdjBuffers bf;
    int rc;
    if ((rc = dev_alloc(&bf.len, (size_t)n * m, fn, "the successor lengths")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.C3, (size_t)m * z * n * ns, fn, "the projection coefficients")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.seg, (size_t)(k + 1) * rn, fn, "the recomputed alphas")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.lamA, rn, fn, "the adjoint")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.lamB, rn, fn, "the adjoint")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.vals, r, fn, "the values")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.V, 1, fn, "the value")) != NOVA_SUCCESS) return rc;
    if ((rc = dev_alloc(&bf.istar, 1, fn, "the maximising alpha")) != NOVA_SUCCESS) return rc;
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;

    adj_len_kernel<<<ceil_div((size_t)n * m, 256), 256>>>(n * m, ns, md.S, bf.len);
    if ((rc = check_launch(fn, "successor lengths")) != NOVA_SUCCESS) return rc;
    adj_coef_kernel<<<std::min<size_t>(ceil_div((size_t)m * z * n * ns, 256), 65535u * 8u), 256>>>(md, bf.len, bf.C3);
    if ((rc = check_launch(fn, "projection coefficients")) != NOVA_SUCCESS) return rc;
    if (cudaMemset(d_dR, 0, (size_t)n * m * sizeof(double)) != cudaSuccess ||
            cudaMemset(d_dT, 0, (size_t)n * m * ns * sizeof(double)) != cudaSuccess ||
            cudaMemset(d_dO, 0, (size_t)m * n * z * sizeof(double)) != cudaSuccess ||
            cudaMemset(bf.lamA, 0, rn * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to clear the gradients.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }

    // Recompute the segment of checkpoint c: seg[q] = Gamma_{ck + q} for
    // q = 0 .. last (last = k - 1, or horizon - ck for the final segment,
    // which also yields Gamma_H).
    auto recompute = [&](unsigned c, unsigned last) -> int {
        const size_t base = (size_t)c * k;
        if (cudaMemcpy(bf.seg, d_checkpoints + (size_t)c * rn, rn * sizeof(float), cudaMemcpyDeviceToDevice) !=
                cudaSuccess) {
            cudaGetLastError();
            NOVA_ERR(fn, "Failed to copy a checkpoint.");
            return NOVA_ERROR_KERNEL_EXECUTION;
        }
        for (unsigned q = 1; q <= last; q++) {
            const size_t step = base + q - 1;
            replay_kernel<<<r, 256, z * sizeof(unsigned)>>>(md, bf.len, bf.C3, bf.seg + (size_t)(q - 1) * rn,
                                                             d_actions + step * r, d_selects + step * r * z,
                                                             bf.seg + (size_t)q * rn);
            int e = check_launch(fn, "alpha recomputation");
            if (e != NOVA_SUCCESS) return e;
        }
        return NOVA_SUCCESS;
    };

    const unsigned nCk = ceil_div(horizon, k);
    unsigned segC = nCk - 1;
    unsigned segStart = segC * k;
    if ((rc = recompute(segC, horizon - segStart)) != NOVA_SUCCESS) return rc;
    const float *GH = bf.seg + (size_t)(horizon - segStart) * rn;
    value_rows_kernel<<<r, 256>>>(GH, n, d_b, bf.vals);
    if ((rc = check_launch(fn, "FP64 values")) != NOVA_SUCCESS) return rc;
    value_argmax_kernel<<<1, 256>>>(r, n, bf.vals, d_b, bf.V, bf.istar, bf.lamA);
    if ((rc = check_launch(fn, "FP64 argmax")) != NOVA_SUCCESS) return rc;

    for (unsigned t = horizon; t >= 1; t--) {
        const unsigned p = t - 1;  // Gamma_{t-1} and the selections of backup t
        if (p < segStart) {
            segC = p / k;
            segStart = segC * k;
            if ((rc = recompute(segC, k - 1)) != NOVA_SUCCESS) return rc;
        }
        if (cudaMemsetAsync(bf.lamB, 0, rn * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            NOVA_ERR(fn, "Failed to clear the adjoint.");
            return NOVA_ERROR_KERNEL_EXECUTION;
        }
        adjoint_step_kernel<<<r, 256, stepSmem>>>(md, bf.len, bf.seg + (size_t)(p - segStart) * rn,
                                                  d_actions + (size_t)p * r, d_selects + (size_t)p * r * z, bf.lamA,
                                                  bf.lamB, d_dR, d_dT, d_dO);
        if ((rc = check_launch(fn, "reverse step")) != NOVA_SUCCESS) return rc;
        std::swap(bf.lamA, bf.lamB);
    }
    if (d_dGamma0 != nullptr &&
            cudaMemcpy(d_dGamma0, bf.lamA, rn * sizeof(double), cudaMemcpyDeviceToDevice) != cudaSuccess) {
        cudaGetLastError();
        NOVA_ERR(fn, "Failed to copy the Gamma_0 gradient.");
        return NOVA_ERROR_KERNEL_EXECUTION;
    }
    if ((rc = sync_device(fn)) != NOVA_SUCCESS) return rc;
    if (Vb != nullptr && (rc = d2h(Vb, bf.V, sizeof(double), fn, "the value")) != NOVA_SUCCESS) return rc;
    if (bestAlpha != nullptr && (rc = d2h(bestAlpha, bf.istar, sizeof(unsigned), fn, "the maximising alpha")) !=
            NOVA_SUCCESS)
        return rc;
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_execute_recorded_gpu(const POMDP *pomdp, POMDPPBVIGPU *pbvi, unsigned int horizon,
                                               unsigned int checkpointEvery, float *d_checkpoints,
                                               unsigned int *d_actions, unsigned int *d_selects) {
    static const char *fn = "pomdp_pbvi_execute_recorded_gpu";
    if (pomdp == nullptr || pbvi == nullptr || horizon == 0 || checkpointEvery == 0 || d_checkpoints == nullptr ||
            d_actions == nullptr || d_selects == nullptr || pbvi->d_Gamma == nullptr || pbvi->d_GammaPrime == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    const size_t rn = (size_t)pomdp->r * pomdp->n;
    for (unsigned t = 0; t < horizon; t++) {
        if (t % checkpointEvery == 0) {
            const float *cur = (pbvi->currentHorizon % 2u == 0u) ? pbvi->d_Gamma : pbvi->d_GammaPrime;
            if (cudaMemcpy(d_checkpoints + (size_t)(t / checkpointEvery) * rn, cur, rn * sizeof(float),
                           cudaMemcpyDeviceToDevice) != cudaSuccess) {
                cudaGetLastError();
                NOVA_ERR(fn, "Failed to store a checkpoint.");
                return NOVA_ERROR_KERNEL_EXECUTION;
            }
        }
        int rc = pomdp_pbvi_update_record_gpu(pomdp, pbvi, d_actions + (size_t)t * pomdp->r,
                                              d_selects + (size_t)t * pomdp->r * pomdp->z);
        if (rc != NOVA_SUCCESS) return rc;
    }
    return NOVA_SUCCESS;
}

extern "C" int pomdp_pbvi_value_replay_f64_gpu(const POMDP *pomdp, unsigned int horizon, const float *d_Gamma0,
                                               const unsigned int *d_actions, const unsigned int *d_selects,
                                               const float *d_b, unsigned int alpha, double *Vb,
                                               unsigned int *bestAlpha) {
    static const char *fn = "pomdp_pbvi_value_replay_f64_gpu";
    if (pomdp == nullptr || pomdp->n == 0 || pomdp->ns == 0 || pomdp->m == 0 || pomdp->z == 0 || pomdp->r == 0 ||
            pomdp->d_S == nullptr || pomdp->d_T == nullptr || pomdp->d_O == nullptr || pomdp->d_R == nullptr ||
            d_Gamma0 == nullptr || (horizon > 0 && (d_actions == nullptr || d_selects == nullptr)) ||
            d_b == nullptr || Vb == nullptr) {
        NOVA_ERR(fn, "Invalid arguments.");
        return NOVA_ERROR_INVALID_DATA;
    }
    AdjModel md{pomdp->n, pomdp->ns, pomdp->m, pomdp->z, pomdp->r, pomdp->gamma,
                pomdp->d_S, pomdp->d_T, pomdp->d_O, pomdp->d_R};
    const unsigned n = md.n, r = md.r, z = md.z, m = md.m, ns = md.ns;
    const size_t rn = (size_t)r * n;
    unsigned *len = nullptr;
    double *GA = nullptr, *GB = nullptr, *vals = nullptr;
    int rc;
    auto cleanup = [&]() {
        cudaDeviceSynchronize();
        cudaFree(len); cudaFree(GA); cudaFree(GB); cudaFree(vals);
    };
    if ((rc = dev_alloc(&len, (size_t)n * m, fn, "the successor lengths")) != NOVA_SUCCESS ||
            (rc = dev_alloc(&GA, rn, fn, "the FP64 alphas")) != NOVA_SUCCESS ||
            (rc = dev_alloc(&GB, rn, fn, "the FP64 alphas")) != NOVA_SUCCESS ||
            (rc = dev_alloc(&vals, r, fn, "the values")) != NOVA_SUCCESS) {
        cleanup();
        return rc;
    }
    adj_len_kernel<<<ceil_div((size_t)n * m, 256), 256>>>(n * m, ns, md.S, len);
    if ((rc = check_launch(fn, "successor lengths")) == NOVA_SUCCESS) {
        widen_kernel<<<(unsigned)std::min<size_t>(ceil_div(rn, 256), 65535u * 8u), 256>>>(d_Gamma0, rn, GA);
        rc = check_launch(fn, "FP64 alphas");
    }
    for (unsigned t = 0; t < horizon && rc == NOVA_SUCCESS; t++) {
        replay_f64_kernel<<<r, 256, z * sizeof(unsigned)>>>(md, len, GA, d_actions + (size_t)t * r,
                                                             d_selects + (size_t)t * r * z, GB);
        rc = check_launch(fn, "FP64 replay");
        std::swap(GA, GB);
    }
    if (rc == NOVA_SUCCESS) {
        value_rows_f64_kernel<<<r, 256>>>(GA, n, d_b, vals);
        rc = check_launch(fn, "FP64 values");
    }
    if (rc == NOVA_SUCCESS) rc = sync_device(fn);
    std::vector<double> hv;
    if (rc == NOVA_SUCCESS) {
        hv.resize(r);
        rc = d2h(hv.data(), vals, r * sizeof(double), fn, "the values");
    }
    cleanup();
    if (rc != NOVA_SUCCESS) return rc;
    // The given alpha, or the maximum from the -1e10 start with the lowest
    // index on ties (pomdp_alpha_vectors.cpp:52-79).
    unsigned best = alpha;
    double V = (double)NOVA_FLT_MIN;
    if (alpha < r) {
        V = hv[alpha];
    } else {
        best = 0;
        for (unsigned i = 0; i < r; i++)
            if (hv[i] > V) { V = hv[i]; best = i; }
    }
    *Vb = V;
    if (bestAlpha != nullptr) *bestAlpha = best;
    return NOVA_SUCCESS;
}
