// pe_objective.cu -- the smoothed tail-aware objective from a forward pass only, in FP32 or FP64.
//
// The quantity pe_grad differentiates (pe_grad_model.h), evaluated without the adjoint: for
// finite differences, line searches, and as the FP64 yardstick of the FP32 gradient on the GPU.
// Unlike the evaluation path (pe_prepare.cu + pe_flight*.cu, the reference's float arithmetic),
// every stage here -- mesh, mass properties, panels, print variation, flight -- runs in the
// chosen precision, so central differences at a step of 1e-4 of a gene's range are not swamped by
// float rounding of the inputs.  Built without fast math.
//
//   k_obj_prepare   one block per plane: mesh, printability, mass properties (two passes over
//                   the triangles with block reductions) and panels, in T.
//   k_obj_forward   one block of kObjW warps per flight, persistent over a work queue: print
//                   variation, staging, release and the flight; writes the smoothed distance.
//   k_obj_weights   one block per plane: the tail-aware objective of its distances.
#include <cuda_runtime.h>

#include "pe_grad_model.h"
#include "pe_internal.cuh"

namespace pe {

namespace {

constexpr int kObjThreads = 128;
constexpr int kObjW = 4;

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Reduction of N values over a block of kObjThreads: op 0 sum, 1 min, 2 max (every thread gets
// the results).
template <class T, int N>
__device__ __forceinline__ void block_reduce(T v[N], const int op[N], T (*scratch)[N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; k++)
        for (int o = 16; o > 0; o >>= 1) {
            const T u = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = op[k] == 0 ? v[k] + u : (op[k] == 1 ? (u < v[k] ? u : v[k]) : (u > v[k] ? u : v[k]));
        }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) scratch[warp][k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) {
        T t = scratch[0][k];
#pragma unroll
        for (int w = 1; w < kObjThreads / 32; w++) {
            const T u = scratch[w][k];
            t = op[k] == 0 ? t + u : (op[k] == 1 ? (u < t ? u : t) : (u > t ? u : t));
        }
        v[k] = t;
    }
    __syncthreads();
}

// ------------------------------------------------------------------ plane data in T
template <class T>
__global__ void __launch_bounds__(kObjThreads) k_obj_prepare(ObjArgs a) {
    using V3T = pg::V3<T>;
    __shared__ T g[kGenomeN];
    __shared__ V3T V[kNvMax];
    __shared__ T red[kObjThreads / 32][8];
    const int p = blockIdx.x, tid = threadIdx.x;
    T* out = reinterpret_cast<T*>(a.plane) + (size_t)p * kObjPlaneStride;
    if (tid < kGenomeN) g[tid] = (T)a.genomes[(size_t)p * kGenomeN + tid];
    __syncthreads();
    const pg::Topo tp = pg::topology(g);
    for (int i = tid; i < tp.nv; i += kObjThreads) V[i] = pg::mesh_vertex(g, tp, i);
    __syncthreads();
    // printability: the mesh extent against the print volume (src/common.h:294-307)
    {
        const T big = T(1e30f);
        T e[6] = {big, big, big, -big, -big, -big};
        for (int i = tid; i < tp.nv; i += kObjThreads) {
            e[0] = pg::p_min(e[0], V[i].x); e[1] = pg::p_min(e[1], V[i].y); e[2] = pg::p_min(e[2], V[i].z);
            e[3] = pg::p_max(e[3], V[i].x); e[4] = pg::p_max(e[4], V[i].y); e[5] = pg::p_max(e[5], V[i].z);
        }
        const int ops[6] = {1, 1, 1, 2, 2, 2};
        block_reduce<T, 6>(e, ops, reinterpret_cast<T(*)[6]>(red));
        const T lim = (T)(0.250f - 0.00045f);
        if (tid == 0)
            out[7] = (e[3] - e[0] <= lim && e[4] - e[1] <= lim && e[5] - e[2] <= lim) ? (T)tp.nt : T(0);
    }
    // mass properties
    T m4[4] = {T(0), T(0), T(0), T(0)};
    for (int i = tid; i < tp.nt; i += kObjThreads) {
        T mi;
        V3T mc;
        pg::tri_mass(V, tp, i, &mi, &mc);
        m4[0] += mi; m4[1] += mc.x; m4[2] += mc.y; m4[3] += mc.z;
    }
    const int sum4[4] = {0, 0, 0, 0};
    block_reduce<T, 4>(m4, sum4, reinterpret_cast<T(*)[4]>(red));
    T m = m4[0], mn;
    V3T c = pg::v3(m4[1], m4[2], m4[3]), np;
    pg::mass_com(g, &m, &c, &mn, &np);
    T I[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    for (int i = tid; i < tp.nt; i += kObjThreads) pg::tri_inertia(V, tp, i, c, I);
    const int sum6[6] = {0, 0, 0, 0, 0, 0};
    block_reduce<T, 6>(I, sum6, reinterpret_cast<T(*)[6]>(red));
    pg::inertia_finish(mn, np, c, I);
    if (tid == 0) {
        out[0] = m;
#pragma unroll
        for (int q = 0; q < 6; q++) out[1 + q] = I[q];
    }
    T* pc = out + 8;
    for (int t = tid; t < tp.nt; t += kObjThreads) {
        V3T ct, n;
        T A;
        pg::panel(V, tp, c, t, &ct, &A, &n);
        pc[t] = ct.x; pc[kNtMax + t] = ct.y; pc[2 * kNtMax + t] = ct.z; pc[3 * kNtMax + t] = A;
        pc[4 * kNtMax + t] = n.x; pc[5 * kNtMax + t] = n.y; pc[6 * kNtMax + t] = n.z;
    }
}

// ------------------------------------------------------------------ flights in T
template <class T>
__global__ void __launch_bounds__(32 * kObjW) k_obj_forward(ObjArgs a) {
    using V3T = pg::V3<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* part = reinterpret_cast<T*>(smem_raw);        // [2][kObjW][8]
    int* flight = reinterpret_cast<int*>(part + 2 * kObjW * 8);
    T* sp = part + 2 * kObjW * 8 + 2;                 // 7 x kNtMax staged panels (SoA)
    constexpr int nthr = 32 * kObjW;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n_flights = a.pop * a.nseeds;
    for (;;) {
        if (tid == 0) *flight = atomicAdd(a.work, 1);
        __syncthreads();
        const int f = *flight;
        __syncthreads();
        if (f >= n_flights) break;
        const int p = f / a.nseeds, si = f - p * a.nseeds;
        const T* pl = reinterpret_cast<const T*>(a.plane) + (size_t)p * kObjPlaneStride;
        const int nt = (int)pl[7];
        if (nt <= 0) {  // does not fit the print volume
            if (tid == 0) a.dist[f] = -100.0;
            continue;
        }
        const int seed = a.seeds[si] + (a.vary ? p * 7919 : 0);
        Scenario S;
        scenario_desc(seed, &S);
        T sc[kScenN];
#pragma unroll
        for (int k = 0; k < kScenN; k++) sc[k] = (T)S.v[k];
        pg::FlightP<T> P;
        V3T cg;
        T sigma, beta[6], I[6];
#pragma unroll
        for (int q = 0; q < 6; q++) I[q] = pl[1 + q];
        pg::printed(sc, pl[0], I, P, &cg, &sigma, beta);
        P.phase = (T)seed_phase(seed);
        const T* pc = pl + 8;
        for (int i = tid; i < nt; i += nthr) {
            V3T rb, nb;
            T ak;
            pg::stage(pg::v3(pc[i], pc[kNtMax + i], pc[2 * kNtMax + i]), pc[3 * kNtMax + i],
                      pg::v3(pc[4 * kNtMax + i], pc[5 * kNtMax + i], pc[6 * kNtMax + i]), cg, sc[pg::SC_RHO],
                      sc[pg::SC_WP], sc[pg::SC_WR], &rb, &nb, &ak);
            sp[i] = rb.x; sp[kNtMax + i] = rb.y; sp[2 * kNtMax + i] = rb.z;
            sp[3 * kNtMax + i] = nb.x; sp[4 * kNtMax + i] = nb.y; sp[5 * kNtMax + i] = nb.z;
            sp[6 * kNtMax + i] = ak;
        }
        pg::St<T> s = pg::release(sc, P, cg, (V3T*)nullptr, (V3T*)nullptr);
        __syncthreads();
        pg::Pre<T> pr;
        pg::step_pre(P, s, pr);
        int par = 0, to_chunk = kChunk;
        for (int j = 0;; j++) {
            T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            for (int i = tid; i < nt; i += nthr) {
                V3T fo, tq;
                pg::panel_fwd(pr, pg::v3(sp[i], sp[kNtMax + i], sp[2 * kNtMax + i]),
                              pg::v3(sp[3 * kNtMax + i], sp[4 * kNtMax + i], sp[5 * kNtMax + i]), sp[6 * kNtMax + i],
                              P.cf, &fo, &tq);
                acc[0] += fo.x; acc[1] += fo.y; acc[2] += fo.z;
                acc[3] += tq.x; acc[4] += tq.y; acc[5] += tq.z;
            }
            T* mine = part + (par * kObjW + warp) * 8;
#pragma unroll
            for (int k = 0; k < 6; k++) acc[k] = warp_sum_t(acc[k]);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 6; k++) mine[k] = acc[k];
            __syncthreads();
            T v[6];
#pragma unroll
            for (int k = 0; k < 6; k++) {
                T t = part[(par * kObjW) * 8 + k];
#pragma unroll
                for (int w = 1; w < kObjW; w++) t += part[(par * kObjW + w) * 8 + k];
                v[k] = t;
            }
            par ^= 1;
            const pg::St<T> nx = pg::step_post(P, s, pr, pg::v3(v[0], v[1], v[2]), pg::v3(v[3], v[4], v[5]));
            T d = T(0);
            int kind = 0;
            if (pg::terminate(s, nx, j, a.max_steps, &d, &kind)) {
                if (tid == 0) a.dist[f] = (double)d;
                break;
            }
            s = nx;
            if (--to_chunk == 0) { s.t = T((double)(j + 1)) * T(pg::kDt); to_chunk = kChunk; }  // src/sim.cu:113
            pg::step_pre(P, s, pr);
        }
    }
}

template <class T>
__global__ void __launch_bounds__(32) k_obj_weights(ObjArgs a) {
    __shared__ T d[kGradMaxSeeds], w[kGradMaxSeeds];
    const int p = blockIdx.x, tid = threadIdx.x, S = a.nseeds;
    for (int s = tid; s < S; s += 32) d[s] = (T)a.dist[(size_t)p * S + s];
    __syncwarp();
    if (tid == 0) a.obj[p] = (double)pg::objective_weights(d, S, w);
}

template <class T>
size_t forward_smem() {
    return (size_t)(2 * kObjW * 8 + 2) * sizeof(T) + (size_t)7 * kNtMax * sizeof(T);
}

template <class T>
cudaError_t launch_t(const ObjArgs& a, int nsm, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(k_obj_forward<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)forward_smem<T>());
    if (e != cudaSuccess) return e;
    int bpsm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, k_obj_forward<T>, 32 * kObjW, forward_smem<T>());
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(a.work, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_obj_prepare<T><<<a.pop, kObjThreads, 0, s>>>(a);
    k_obj_forward<T><<<(bpsm > 0 ? bpsm : 1) * nsm, 32 * kObjW, forward_smem<T>(), s>>>(a);
    if (a.obj) k_obj_weights<T><<<a.pop, 32, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_objective(const ObjArgs& a, int precision, int nsm, cudaStream_t s) {
    return precision == 64 ? launch_t<double>(a, nsm, s) : launch_t<float>(a, nsm, s);
}

}  // namespace pe
