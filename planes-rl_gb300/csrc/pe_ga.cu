// pe_ga.cu -- the GA on the device and the hybrid search (GA + Adam on the adjoint gradient).
//
// The operators and their constants are the reference's run_ga (src/sim.cu:472-489): the best
// pop/64 genomes carry over, 5 % of children are fresh draws, the rest blend two 4-way
// tournament winners gene by gene (a ~ U(-0.1, 1.1)) and mutate a gene with probability 0.25 by
// N(0, 1) * 0.08 * range * anneal, anneal = 1 - 0.6 gen / gens, then clamp to the bounds.  Only
// the random stream differs: a counter-based SplitMix64 hash keyed by (seed, generation, child,
// draw) instead of one std::mt19937, so a generation is one kernel and the genomes stay in HBM.
// The host GA (pe_run_ga) keeps the reference's stream and is the parity mode.
//
// Kernels:
//   k_topk      one block: the k best scores exactly (radix select on the ordered float bits,
//               ties to the lower index), sorted best first by a bitonic sort in shared memory.
//   k_ga_next   one thread per child of the next generation.
//   k_adam      one thread per (genome, gene): an Adam ascent step in normalized genome units.
//   k_gather / k_scatter   rows of a population by index.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#include "../../include/planes_eval.h"
#include "pe_internal.cuh"

namespace pe {
namespace {

__constant__ float c_lo[kGenomeN], c_hi[kGenomeN];

// SplitMix64 finalizer (Steele, Lea and Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014), used as a hash of (key, draw index).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
struct Stream {
    uint64_t key;
    uint32_t n;
    __device__ Stream(uint64_t seed, uint32_t gen, uint32_t child)
        : key(mix64(mix64(seed) ^ ((uint64_t)gen << 32 | child))), n(0) {}
    __device__ __forceinline__ float u01() {  // [0, 1), 24 bits
        return (float)(mix64(key ^ (uint64_t)(n++) * 0xD1B54A32D192ED03ull) >> 40) * (1.0f / 16777216.0f);
    }
    __device__ __forceinline__ float normal() {  // Box-Muller
        const float u1 = 1.0f - u01(), u2 = u01();
        return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    }
};

__device__ __forceinline__ float clamp_gene(int j, float v) { return fminf(c_hi[j], fmaxf(c_lo[j], v)); }

// float -> uint32 in the same order (NaN lowest)
__device__ __forceinline__ uint32_t order_key(float f) {
    if (f != f) return 0u;
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

constexpr int kTopThreads = 1024;
constexpr int kTopMax = 4096;

__global__ void __launch_bounds__(kTopThreads) k_topk(const float* score, int n, int k, int* out_idx,
                                                      float* out_score) {
    __shared__ uint32_t hist[256];
    __shared__ uint32_t s_prefix, s_need, s_count;
    __shared__ uint32_t skey[kTopMax];
    __shared__ int sidx[kTopMax];
    __shared__ int wsum[kTopThreads / 32];
    const int tid = threadIdx.x;
    if (tid == 0) { s_prefix = 0; s_need = (uint32_t)k; s_count = 0; }
    uint32_t mask = 0;
    // radix select of the k-th largest key, 8 bits at a time
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int b = tid; b < 256; b += kTopThreads) hist[b] = 0;
        __syncthreads();
        const uint32_t prefix = s_prefix;
        for (int i = tid; i < n; i += kTopThreads) {
            const uint32_t key = order_key(score[i]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t need = s_need, cum = 0;
            int b = 255;
            for (; b > 0; b--) {
                if (cum + hist[b] >= need) break;
                cum += hist[b];
            }
            s_need = need - cum;
            s_prefix = prefix | ((uint32_t)b << shift);
        }
        mask |= 255u << shift;
        __syncthreads();
    }
    const uint32_t kth = s_prefix;
    const uint32_t ties = s_need;  // how many keys equal to kth make the cut
    // everything above the k-th key (order of arrival; sorted below)
    for (int i = tid; i < n; i += kTopThreads) {
        const uint32_t key = order_key(score[i]);
        if (key > kth) {
            const uint32_t at = atomicAdd(&s_count, 1u);
            skey[at] = key;
            sidx[at] = i;
        }
    }
    __syncthreads();
    // the lowest-index ties, chunk by chunk in index order
    uint32_t taken = 0;
    const int lane = tid & 31, warp = tid >> 5;
    for (int c0 = 0; c0 < n && taken < ties; c0 += kTopThreads) {
        const int i = c0 + tid;
        const bool tie = i < n && order_key(score[i]) == kth;
        const unsigned bal = __ballot_sync(0xffffffffu, tie);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < kTopThreads / 32; w++) {
            if (w < warp) before += wsum[w];
            total += wsum[w];
        }
        const int rank = before + __popc(bal & ((1u << lane) - 1u));
        const uint32_t base = (uint32_t)k - ties;
        if (tie && taken + (uint32_t)rank < ties) {
            skey[base + taken + rank] = kth;
            sidx[base + taken + rank] = i;
        }
        taken += (uint32_t)total;
        __syncthreads();
    }
    // bitonic sort of the k candidates: key descending, index ascending
    int m = 1;
    while (m < k) m <<= 1;
    for (int i = k + tid; i < m; i += kTopThreads) { skey[i] = 0u; sidx[i] = 0x7fffffff; }
    __syncthreads();
    for (int size = 2; size <= m; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < m; i += kTopThreads) {
                const int jx = i ^ stride;
                if (jx > i) {
                    // "before" = better: larger key, then smaller index
                    const bool better_j = skey[jx] > skey[i] || (skey[jx] == skey[i] && sidx[jx] < sidx[i]);
                    const bool up = (i & size) == 0;
                    if (up == better_j) {
                        const uint32_t tk = skey[i]; skey[i] = skey[jx]; skey[jx] = tk;
                        const int ti = sidx[i]; sidx[i] = sidx[jx]; sidx[jx] = ti;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = tid; i < k; i += kTopThreads) {
        out_idx[i] = sidx[i];
        if (out_score) out_score[i] = score[sidx[i]];
    }
}

__global__ void k_ga_next(const float* genomes, const float* score, const int* top, int pop, int elite, int gen,
                          int gens, uint64_t seed, float* next) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pop) return;
    float* out = next + (size_t)i * kGenomeN;
    if (i < elite) {
        const float* src = genomes + (size_t)top[i] * kGenomeN;
        for (int j = 0; j < kGenomeN; j++) out[j] = src[j];
        return;
    }
    Stream r(seed, (uint32_t)gen, (uint32_t)i);
    if (r.u01() < 0.05f) {  // fresh draw
        for (int j = 0; j < kGenomeN; j++) out[j] = clamp_gene(j, c_lo[j] + r.u01() * (c_hi[j] - c_lo[j]));
        return;
    }
    auto tournament = [&]() {
        int b = min((int)(r.u01() * pop), pop - 1);
        for (int t = 0; t < 3; t++) {
            const int c = min((int)(r.u01() * pop), pop - 1);
            if (score[c] > score[b]) b = c;
        }
        return b;
    };
    const float* pa = genomes + (size_t)tournament() * kGenomeN;
    const float* pc = genomes + (size_t)tournament() * kGenomeN;
    const float anneal = 1.0f - 0.6f * gen / gens;
    for (int j = 0; j < kGenomeN; j++) {
        const float a = -0.1f + 1.2f * r.u01();
        float v = pa[j] * a + pc[j] * (1.0f - a);
        if (r.u01() < 0.25f) v += r.normal() * 0.08f * (c_hi[j] - c_lo[j]) * anneal;
        out[j] = clamp_gene(j, v);
    }
}

__global__ void k_gather(const float* src, const int* idx, int n, float* dst) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * kGenomeN) dst[t] = src[(size_t)idx[t / kGenomeN] * kGenomeN + t % kGenomeN];
}
__global__ void k_scatter(const float* src, const float* src_score, const int* idx, int n, float* dst,
                          float* dst_score) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * kGenomeN) dst[(size_t)idx[t / kGenomeN] * kGenomeN + t % kGenomeN] = src[t];
    if (t < n && dst_score) dst_score[idx[t]] = src_score[t];
}

// Adam ascent in normalized units x = (g - lo) / (hi - lo): dJ/dx = dJ/dg (hi - lo).
__global__ void k_adam(float* g, const float* grad, float* m, float* v, int n, int t, float lr) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n * kGenomeN) return;
    const int j = k % kGenomeN;
    const float range = c_hi[j] - c_lo[j];
    const float gx = grad[k] * range;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mk = b1 * m[k] + (1.0f - b1) * gx, vk = b2 * v[k] + (1.0f - b2) * gx * gx;
    m[k] = mk;
    v[k] = vk;
    const float mh = mk / (1.0f - powf(b1, (float)t)), vh = vk / (1.0f - powf(b2, (float)t));
    const float x = (g[k] - c_lo[j]) / range + lr * mh / (sqrtf(vh) + eps);
    g[k] = clamp_gene(j, c_lo[j] + fminf(1.0f, fmaxf(0.0f, x)) * range);
}

}  // namespace
}  // namespace pe

using namespace pe;

namespace {
struct Buf {
    void* p = nullptr;
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes); }
    template <class T> T* as() const { return (T*)p; }
};
// Events released on every return path.
struct Events {
    std::vector<cudaEvent_t> ev;
    ~Events() { for (cudaEvent_t e : ev) if (e) cudaEventDestroy(e); }
    cudaError_t add(cudaEvent_t* out) {
        cudaEvent_t e = nullptr;
        cudaError_t r = cudaEventCreate(&e);
        if (r == cudaSuccess) ev.push_back(e);
        *out = e;
        return r;
    }
};
#define GA_CUDA(x)                                                                          \
    do {                                                                                    \
        cudaError_t e_ = (x);                                                               \
        if (e_ != cudaSuccess) {                                                            \
            (void)cudaGetLastError(); /* reported here: not left pending for the next call */ \
            char m_[256];                                                                   \
            snprintf(m_, sizeof m_, "%s: %s", #x, cudaGetErrorString(e_));                  \
            pe::set_last_error(m_);                                                         \
            return PE_ECUDA;                                                                \
        }                                                                                   \
    } while (0)
#define GA_PE(x)                          \
    do {                                  \
        int r_ = (x);                     \
        if (r_ != PE_OK) return r_;       \
    } while (0)
}  // namespace

extern "C" int pe_topk(const float* d_scores, int n, int k, int* d_idx, float* d_top, void* stream) {
    if (!d_scores || !d_idx) { set_last_error("NULL scores or index output"); return PE_EINVAL; }
    if (n < 1 || k < 1 || k > n || k > kTopMax) { set_last_error("pe_topk needs 1 <= k <= min(n, 4096)"); return PE_EINVAL; }
    k_topk<<<1, kTopThreads, 0, (cudaStream_t)stream>>>(d_scores, n, k, d_idx, d_top);
    GA_CUDA(cudaGetLastError());
    return PE_OK;
}

extern "C" int pe_select_top(const float* d_genomes, const float* d_scores, int pop, int k, float* d_top,
                             int* d_idx, void* stream) {
    if (!d_genomes || !d_scores || !d_top || !d_idx) { set_last_error("NULL argument"); return PE_EINVAL; }
    if (pop < 1 || k < 1 || k > pop || k > kTopMax) { set_last_error("pe_select_top needs 1 <= k <= min(pop, 4096)"); return PE_EINVAL; }
    const cudaStream_t s = (cudaStream_t)stream;
    k_topk<<<1, kTopThreads, 0, s>>>(d_scores, pop, k, d_idx, nullptr);
    k_gather<<<(k * kGenomeN + 255) / 256, 256, 0, s>>>(d_genomes, d_idx, k, d_top);
    GA_CUDA(cudaGetLastError());
    return PE_OK;
}

static int upload_bounds() {
    float lo[kGenomeN], hi[kGenomeN];
    pe_genome_bounds(lo, hi);
    GA_CUDA(cudaMemcpyToSymbol(c_lo, lo, sizeof lo));
    GA_CUDA(cudaMemcpyToSymbol(c_hi, hi, sizeof hi));
    return PE_OK;
}

extern "C" int pe_ga_step(const float* d_genomes, const float* d_scores, int pop, int gen, int gens,
                          unsigned long long seed, float* d_next, void* stream) {
    if (!d_genomes || !d_scores || !d_next || d_next == d_genomes) {
        set_last_error("NULL or aliased genome buffers");
        return PE_EINVAL;
    }
    if (pop < 64 || pop / 64 > kTopMax || gens < 1 || gen < 0) {
        set_last_error("pe_ga_step needs 64 <= pop <= 262144 and 0 <= gen < gens");
        return PE_EINVAL;
    }
    GA_PE(upload_bounds());
    const int elite = pop / 64;
    int* d_top = nullptr;
    GA_CUDA(cudaMallocAsync((void**)&d_top, sizeof(int) * elite, (cudaStream_t)stream));
    k_topk<<<1, kTopThreads, 0, (cudaStream_t)stream>>>(d_scores, pop, elite, d_top, nullptr);
    k_ga_next<<<(pop + 127) / 128, 128, 0, (cudaStream_t)stream>>>(d_genomes, d_scores, d_top, pop, elite, gen, gens,
                                                                  (uint64_t)seed, d_next);
    cudaError_t err = cudaGetLastError();
    cudaFreeAsync(d_top, (cudaStream_t)stream);
    GA_CUDA(err);
    return PE_OK;
}

extern "C" int pe_evolve(pe_engine* e, const pe_evolve_config* cfg, float* h_history, pe_evolve_result* out) {
    if (!e || !cfg || !out) { set_last_error("NULL engine, config or result"); return PE_EINVAL; }
    const pe_evolve_config c = *cfg;
    if (c.pop < 64 || c.gens < 1 || c.nseeds < 1 || c.nseeds > 256 || c.max_steps < 1 || c.max_steps > kMaxSteps ||
        c.polish_top < 0 || c.polish_top > c.pop || c.polish_steps < 0 || c.holdout < 0 || c.holdout > 4096 ||
        c.audit < 0 || c.audit > 4096 || c.polish_max_steps < 0 || c.polish_max_steps > kMaxSteps) {
        set_last_error("pe_evolve: pop >= 64, gens >= 1, 1 <= nseeds <= 256, steps <= 7200, holdout/audit <= 4096");
        return PE_EINVAL;
    }
    const int pop = c.pop, S = c.nseeds, G = kGenomeN;
    const int elite = pop / 64;
    const int n_hold = c.holdout > 0 ? std::min(8, pop) : 0;
    const int k_sel = std::max(std::max(elite, std::max(c.polish_top, n_hold)), 1);
    if (k_sel > kTopMax) { set_last_error("pe_evolve: pop / 64 and polish_top must be <= 4096"); return PE_EINVAL; }
    GA_PE(upload_bounds());
    std::vector<float> h_g((size_t)pop * G);
    GA_PE(pe_random_genomes(c.seed, pop, h_g.data()));
    Buf gA, gB, score, dist, top, topsc, pg, pgrad, pm, pv, pscore, pdist, hg, hdist, hsc;
    GA_CUDA(gA.alloc(sizeof(float) * pop * G));
    GA_CUDA(gB.alloc(sizeof(float) * pop * G));
    GA_CUDA(score.alloc(sizeof(float) * pop));
    GA_CUDA(dist.alloc(sizeof(float) * pop * S));
    GA_CUDA(top.alloc(sizeof(int) * k_sel));
    GA_CUDA(topsc.alloc(sizeof(float) * k_sel));
    const int P = std::max(c.polish_top, 1);
    GA_CUDA(pg.alloc(sizeof(float) * P * G));
    GA_CUDA(pgrad.alloc(sizeof(float) * P * G));
    GA_CUDA(pm.alloc(sizeof(float) * P * G));
    GA_CUDA(pv.alloc(sizeof(float) * P * G));
    GA_CUDA(pscore.alloc(sizeof(float) * P));
    GA_CUDA(pdist.alloc(sizeof(float) * P * S));
    const int HN = std::max(n_hold, 1), HS = std::max(c.holdout, 1);
    GA_CUDA(hg.alloc(sizeof(float) * HN * G));
    GA_CUDA(hdist.alloc(sizeof(float) * HN * HS));
    GA_CUDA(hsc.alloc(sizeof(float) * HN));
    GA_CUDA(cudaMemcpy(gA.p, h_g.data(), sizeof(float) * pop * G, cudaMemcpyHostToDevice));
    float* cur = gA.as<float>();
    float* nxt = gB.as<float>();
    std::vector<int> hseeds(c.holdout);
    for (int i = 0; i < c.holdout; i++) hseeds[i] = c.holdout_base + i * 7919;
    std::vector<int> seeds(S);
    std::vector<float> h_sc(pop), h_top(k_sel), h_hsc(HN);
    std::vector<int> h_topi(k_sel);
    float best = -1e30f;
    std::vector<float> best_g(G, 0.f);
    int best_gen = -1;
    Events events;
    cudaEvent_t t0, t1;
    GA_CUDA(events.add(&t0));
    GA_CUDA(events.add(&t1));
    std::vector<cudaEvent_t> gen_end(c.gens, nullptr);
    for (auto& ev : gen_end) GA_CUDA(events.add(&ev));
    GA_CUDA(cudaEventRecord(t0, nullptr));
    int grad_calls = 0;
    for (int gen = 0; gen < c.gens; gen++) {
        for (int s = 0; s < S; s++) seeds[s] = gen * S + s + 1;  // src/sim.cu:435
        GA_PE(pe_eval_batch(e, cur, pop, seeds.data(), S, 0, c.max_steps, dist.as<float>(), nullptr,
                            score.as<float>(), nullptr));
        if (c.polish_top > 0 && c.polish_steps > 0) {
            // Adam on the top polish_top genomes, then their new scores replace the old ones
            k_topk<<<1, kTopThreads>>>(score.as<float>(), pop, c.polish_top, top.as<int>(), nullptr);
            const int nb = (c.polish_top * G + 255) / 256;
            k_gather<<<nb, 256>>>(cur, top.as<int>(), c.polish_top, pg.as<float>());
            GA_CUDA(cudaMemsetAsync(pm.p, 0, sizeof(float) * P * G, nullptr));
            GA_CUDA(cudaMemsetAsync(pv.p, 0, sizeof(float) * P * G, nullptr));
            for (int t = 1; t <= c.polish_steps; t++) {
                GA_PE(pe_grad(e, pg.as<float>(), c.polish_top, seeds.data(), S, 0,
                              c.polish_max_steps > 0 ? c.polish_max_steps : c.max_steps, 60, nullptr,
                              pgrad.as<float>(), nullptr, nullptr));
                grad_calls++;
                k_adam<<<nb, 256>>>(pg.as<float>(), pgrad.as<float>(), pm.as<float>(), pv.as<float>(), c.polish_top,
                                    t, c.polish_lr);
            }
            GA_PE(pe_eval_batch(e, pg.as<float>(), c.polish_top, seeds.data(), S, 0, c.max_steps, pdist.as<float>(),
                                nullptr, pscore.as<float>(), nullptr));
            k_scatter<<<nb, 256>>>(pg.as<float>(), pscore.as<float>(), top.as<int>(), c.polish_top, cur,
                                   score.as<float>());
            GA_CUDA(cudaGetLastError());
        }
        k_topk<<<1, kTopThreads>>>(score.as<float>(), pop, k_sel, top.as<int>(), topsc.as<float>());
        GA_CUDA(cudaGetLastError());
        // holdout of the top 8 (src/sim.cu:446-456); the best-ever genome is chosen by it
        float holdout = -1e30f;
        int champ = 0;
        if (n_hold > 0) {
            k_gather<<<(n_hold * G + 255) / 256, 256>>>(cur, top.as<int>(), n_hold, hg.as<float>());
            GA_PE(pe_eval_batch(e, hg.as<float>(), n_hold, hseeds.data(), c.holdout, 0, c.max_steps,
                                hdist.as<float>(), nullptr, hsc.as<float>(), nullptr));
            GA_CUDA(cudaMemcpy(h_hsc.data(), hsc.p, sizeof(float) * n_hold, cudaMemcpyDeviceToHost));
            for (int q = 0; q < n_hold; q++)
                if (h_hsc[q] > holdout) { holdout = h_hsc[q]; champ = q; }
        }
        GA_CUDA(cudaMemcpy(h_topi.data(), top.p, sizeof(int) * k_sel, cudaMemcpyDeviceToHost));
        if (h_history || n_hold > 0) GA_CUDA(cudaMemcpy(h_sc.data(), score.p, sizeof(float) * pop, cudaMemcpyDeviceToHost));
        if (n_hold > 0 && holdout > best) {
            best = holdout;
            best_gen = gen;
            GA_CUDA(cudaMemcpy(best_g.data(), cur + (size_t)h_topi[champ] * G, sizeof(float) * G, cudaMemcpyDeviceToHost));
        }
        if (h_history) {
            std::vector<float> srt(h_sc);
            std::sort(srt.begin(), srt.end(), [](float a, float b) { return a > b; });
            double mean = 0;
            for (float v : h_sc) mean += v / pop;
            float* hrow = h_history + (size_t)gen * 5;
            hrow[0] = srt[0]; hrow[1] = holdout; hrow[2] = (float)mean; hrow[3] = srt[pop / 10];
        }
        // next generation
        k_ga_next<<<(pop + 127) / 128, 128>>>(cur, score.as<float>(), top.as<int>(), pop, elite, gen, c.gens,
                                              (uint64_t)c.seed, nxt);
        GA_CUDA(cudaGetLastError());
        GA_CUDA(cudaEventRecord(gen_end[gen], nullptr));
        std::swap(cur, nxt);
    }
    GA_CUDA(cudaEventRecord(t1, nullptr));
    GA_CUDA(cudaEventSynchronize(t1));
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    for (int gen = 0; gen < c.gens; gen++) {
        float gms = 0;
        cudaEventElapsedTime(&gms, t0, gen_end[gen]);
        if (h_history) h_history[(size_t)gen * 5 + 4] = gms / 1e3f;
    }
    out->gpu_seconds = ms / 1e3;
    out->best_holdout = best;
    out->best_gen = best_gen;
    out->grad_calls = grad_calls;
    memcpy(out->best_genome, best_g.data(), sizeof(float) * G);
    out->audit_score = 0.f;
    if (c.audit > 0 && best_gen >= 0) {  // the champion on independent scenarios
        std::vector<int> aseeds(c.audit);
        for (int i = 0; i < c.audit; i++) aseeds[i] = c.audit_base + i * 7919;
        float sc = 0;
        GA_PE(pe_evaluate_population(e, best_g.data(), 1, aseeds.data(), c.audit, 0, c.max_steps, nullptr, nullptr,
                                     &sc));
        out->audit_score = sc;
    }
    return PE_OK;
}
