// pe_audit.cu -- the robustness audit's statistics on the device (src/sim.cu:291-309, percentile
// src/sim.cu:250-256): min, p05, p10, p25, median, mean, sd, p75, p90, p95, max, CVaR10 and the
// failure count of n landing distances.
//
// The reference sorts the distances on the host and sums x / n, x^2 / n and (for CVaR10, the mean
// of the worst tenth) x / tail in ascending order, in float.  Here the sort is a bitonic network
// in HBM (blocks of 1024 keys sorted and merged in shared memory, the wider strides one launch
// each), every term x / n, x * x / n and x / tail is formed by its own thread with IEEE-rounded
// intrinsics, and one thread adds the terms in ascending order: the same operations in the same
// order, so each statistic equals the reference's host result bit for bit.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include "../../include/planes_eval.h"
#include "pe_internal.cuh"

namespace pe {
namespace {

constexpr int kSortBlock = 1024;  // keys per block-local sort / merge (512 threads)

__global__ void k_pad_copy(const float* src, int n, int n2, float* keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n2) keys[i] = i < n ? src[i] : INFINITY;
}

__device__ __forceinline__ void cmp_swap(float* a, float* b, bool ascending) {
    const float x = *a, y = *b;
    if ((x > y) == ascending) { *a = y; *b = x; }
}

// Stages j = jmax .. 1 of merge size k (k <= 1024: the whole sort up to k) on one 1024-key block.
// The direction of a pair follows its global index, as in the full network.
__global__ void __launch_bounds__(kSortBlock / 2) k_bitonic_block(float* keys, int kmin, int kmax) {
    __shared__ float s[kSortBlock];
    const int base = blockIdx.x * kSortBlock, t = threadIdx.x;
    s[t] = keys[base + t];
    s[t + kSortBlock / 2] = keys[base + t + kSortBlock / 2];
    __syncthreads();
    for (int k = kmin; k <= kmax; k <<= 1) {
        for (int j = min(k, kSortBlock) >> 1; j > 0; j >>= 1) {
            const int i = (t / j) * 2 * j + (t % j);
            cmp_swap(&s[i], &s[i + j], ((base + i) & k) == 0);
            __syncthreads();
        }
    }
    keys[base + t] = s[t];
    keys[base + t + kSortBlock / 2] = s[t + kSortBlock / 2];
}

// One stage (merge size k, stride j >= 1024) across the whole array: one thread per pair.
__global__ void k_bitonic_stride(float* keys, int n2, int k, int j) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n2 / 2) return;
    const int i = (t / j) * 2 * j + (t % j);
    cmp_swap(&keys[i], &keys[i + j], (i & k) == 0);
}

// terms[0][i] = x / n, terms[1][i] = x * x / n, terms[2][i] = x / tail (i < tail)
__global__ void k_audit_terms(const float* sorted, int n, int tail, float* terms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = sorted[i], fn = (float)n;
    terms[i] = __fdiv_rn(x, fn);
    terms[n + i] = __fdiv_rn(__fmul_rn(x, x), fn);
    if (i < tail) terms[2 * n + i] = __fdiv_rn(x, (float)tail);
}

// src/sim.cu:250-256: linear interpolation between the neighbouring order statistics
__device__ float percentile_sorted(const float* s, int n, float q) {
    const float x = __fmul_rn(q, (float)(n - 1));
    const int a = (int)floorf(x), b = (int)ceilf(x);
    const float t = __fsub_rn(x, (float)a);
    return __fadd_rn(__fmul_rn(s[a], __fsub_rn(1.0f, t)), __fmul_rn(s[b], t));
}

// Thread 0 adds the mean and mean-square terms, thread 32 the CVaR10 terms, thread 64 counts
// failures (distance < 0); thread 0 then writes all 13 statistics.
__global__ void k_audit_sums(const float* sorted, const float* terms, int n, int tail, float* stats) {
    __shared__ float s_cvar;
    __shared__ int s_fail;
    const int t = threadIdx.x;
    if (t == 32) {
        float c = 0.0f;
        for (int i = 0; i < tail; i++) c = __fadd_rn(c, terms[2 * n + i]);
        s_cvar = c;
    } else if (t == 64) {
        int f = 0;
        for (int i = 0; i < n && sorted[i] < 0.0f; i++) f++;  // ascending: the negatives lead
        s_fail = f;
    }
    float mean = 0.0f, sq = 0.0f;
    if (t == 0)
        for (int i = 0; i < n; i++) {
            mean = __fadd_rn(mean, terms[i]);
            sq = __fadd_rn(sq, terms[n + i]);
        }
    __syncthreads();
    if (t != 0) return;
    const float sd = __fsqrt_rn(fmaxf(0.0f, __fsub_rn(sq, __fmul_rn(mean, mean))));
    stats[0] = sorted[0];
    stats[1] = percentile_sorted(sorted, n, .05f);
    stats[2] = percentile_sorted(sorted, n, .10f);
    stats[3] = percentile_sorted(sorted, n, .25f);
    stats[4] = percentile_sorted(sorted, n, .50f);
    stats[5] = mean;
    stats[6] = sd;
    stats[7] = percentile_sorted(sorted, n, .75f);
    stats[8] = percentile_sorted(sorted, n, .90f);
    stats[9] = percentile_sorted(sorted, n, .95f);
    stats[10] = sorted[n - 1];
    stats[11] = s_cvar;
    stats[12] = (float)s_fail;
}

}  // namespace

void set_last_error(const char* msg);  // pe_api.cu

}  // namespace pe

using namespace pe;

extern "C" int pe_distance_stats(const float* d_dist, int n, float* d_stats, void* stream) {
    if (!d_dist || !d_stats) { set_last_error("pe_distance_stats: NULL distances or statistics"); return PE_EINVAL; }
    if (n < 1 || n > (1 << 26)) { set_last_error("pe_distance_stats needs 1 <= n <= 2^26"); return PE_EINVAL; }
    const cudaStream_t s = (cudaStream_t)stream;
    int n2 = kSortBlock;
    while (n2 < n) n2 <<= 1;
    const int tail = n / 10 > 1 ? n / 10 : 1;
    float* keys = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&keys, sizeof(float) * ((size_t)n2 + 3 * (size_t)n), s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_last_error("pe_distance_stats: scratch allocation failed");
        return PE_ECUDA;
    }
    float* terms = keys + n2;
    k_pad_copy<<<(n2 + 255) / 256, 256, 0, s>>>(d_dist, n, n2, keys);
    k_bitonic_block<<<n2 / kSortBlock, kSortBlock / 2, 0, s>>>(keys, 2, kSortBlock);
    for (int k = 2 * kSortBlock; k <= n2; k <<= 1) {
        for (int j = k >> 1; j >= kSortBlock; j >>= 1)
            k_bitonic_stride<<<(n2 / 2 + 255) / 256, 256, 0, s>>>(keys, n2, k, j);
        k_bitonic_block<<<n2 / kSortBlock, kSortBlock / 2, 0, s>>>(keys, k, k);
    }
    k_audit_terms<<<(n + 255) / 256, 256, 0, s>>>(keys, n, tail, terms);
    k_audit_sums<<<1, 96, 0, s>>>(keys, terms, n, tail, d_stats);
    e = cudaGetLastError();
    cudaFreeAsync(keys, s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        char m[160];
        snprintf(m, sizeof m, "pe_distance_stats: %s", cudaGetErrorString(e));
        set_last_error(m);
        return PE_ECUDA;
    }
    return PE_OK;
}
