// pe_scores.cu -- tail-aware fitness per plane (src/sim.cu:340-357):
//   score = 0.65 * mean + 0.25 * mean(worst ceil(S/4)) + 0.10 * worst.
// The reference reduces on the host in IEEE float without contraction; the intrinsics below
// (__fdiv_rn, __fadd_rn, __fmul_rn) reproduce that rounding bit for bit, independent of the
// -use_fast_math this file is built with.  The mean runs in scenario order, the tail in
// ascending order, as std::sort leaves it.
#include "pe_internal.cuh"

namespace pe {

constexpr int kSmallS = 32;     // thread per plane up to this many scenarios
constexpr int kBlockSortS = 4096;  // block per plane (bitonic sort in shared memory) up to this

__device__ __forceinline__ float score_from_sorted_tail(float mean, const float* sorted, int S, int stride) {
    const int tail_n = (S + 3) / 4;
    const float tn = (float)tail_n;
    float cvar = 0.0f;
    for (int s = 0; s < tail_n; s++) cvar = __fadd_rn(cvar, __fdiv_rn(sorted[s * stride], tn));
    return __fadd_rn(__fadd_rn(__fmul_rn(0.65f, mean), __fmul_rn(0.25f, cvar)), __fmul_rn(0.10f, sorted[0]));
}

__global__ void k_scores_small(const float* __restrict__ dist, int pop, int S, float* __restrict__ scores) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pop) return;
    float row[kSmallS];
    const float* d = dist + (size_t)p * S;
    const float fs = (float)S;
    float mean = 0.0f;
    for (int s = 0; s < S; s++) {
        float x = d[s];
        mean = __fadd_rn(mean, __fdiv_rn(x, fs));
        // insertion sort, ascending
        int k = s;
        while (k > 0 && row[k - 1] > x) { row[k] = row[k - 1]; k--; }
        row[k] = x;
    }
    scores[p] = score_from_sorted_tail(mean, row, S, 1);
}

// One block per plane: load, bitonic sort in shared memory (+inf padding), thread 0 sums.
__global__ void __launch_bounds__(1024) k_scores_block(const float* __restrict__ dist, int pop, int S,
                                                       float* __restrict__ scores) {
    extern __shared__ float sh[];
    const int p = blockIdx.x;
    int n = 1;
    while (n < S) n <<= 1;
    const float* d = dist + (size_t)p * S;
    for (int i = threadIdx.x; i < n; i += blockDim.x) sh[i] = i < S ? d[i] : __int_as_float(0x7f800000);
    __syncthreads();
    for (int k = 2; k <= n; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                int l = i ^ jj;
                if (l > i) {
                    float x = sh[i], y = sh[l];
                    bool asc = (i & k) == 0;
                    if ((x > y) == asc) { sh[i] = y; sh[l] = x; }
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        const float fs = (float)S;
        float mean = 0.0f;
        for (int s = 0; s < S; s++) mean = __fadd_rn(mean, __fdiv_rn(d[s], fs));
        scores[p] = score_from_sorted_tail(mean, sh, S, 1);
    }
}

cudaError_t launch_scores(const float* dist, int pop, int S, float* scores, cudaStream_t s) {
    if (pop <= 0) return cudaSuccess;
    if (S <= 0 || S > kBlockSortS) return cudaErrorInvalidValue;
    if (S <= kSmallS) {
        k_scores_small<<<(pop + 127) / 128, 128, 0, s>>>(dist, pop, S, scores);
    } else {
        int n = 1;
        while (n < S) n <<= 1;
        int threads = n < 1024 ? n : 1024;
        k_scores_block<<<pop, threads, n * sizeof(float), s>>>(dist, pop, S, scores);
    }
    return cudaGetLastError();
}

}  // namespace pe
