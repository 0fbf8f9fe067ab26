// pe_prepare.cu -- genome -> mesh -> mass properties -> packed panels (src/sim.cu:25-49).
//
// Three launches:
//   k_topo_scan   triangle count of each genome from its topology genes alone, block-local
//                 exclusive scan, block totals out.
//   k_scan_tot    exclusive scan of the block totals (one block, 1024 at a time); also the
//                 grand total.
//   k_mesh        one warp per plane: lanes evaluate the mesh vertices in parallel into shared
//                 memory and every triangle's mass-property terms likewise; lane 0 adds the terms
//                 in emission order (the reference's order, so the sums round identically); lanes
//                 write the COM-relative panel SoA into the plane's exact prefix range.
// HBM traffic is small (140 B genome in, 32 B per panel out); the cost is lane 0's ordered
// additions, about 1 ms per 100k planes.
#include "pe_internal.cuh"

namespace pe {

__global__ void __launch_bounds__(kScanBlock) k_topo_scan(PrepArgs a) {
    __shared__ int warp_tot[kScanBlock / 32];
    int p = blockIdx.x * kScanBlock + threadIdx.x;
    int n = 0;
    if (p < a.pop) {
        GenomeRef g{a.genomes + (size_t)p * kGenomeN};
        n = topology(g).nt;
        a.nt_topo[p] = n;
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = n;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    int excl = x - n + (w > 0 ? warp_tot[w - 1] : 0);
    if (p < a.pop) a.pt.off[p] = excl;  // block-local for now
    if (threadIdx.x == kScanBlock - 1) a.block_sum[blockIdx.x] = excl + n;
}

// Exclusive scan of nblocks block totals in place, in tiles of 1024 with the running sum of the
// earlier tiles carried through shared memory (PE_MAX_POP planes are 4,096 tiles); grand total to
// *total.  One block: the tiles follow one another.
__global__ void __launch_bounds__(1024) k_scan_tot(int* block_sum, int nblocks, int* total) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += 1024) {
        const int i = base + threadIdx.x;
        const int n = i < nblocks ? block_sum[i] : 0;
        int x = n;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int c = carry;
        const int excl = c + x - n + (w > 0 ? warp_tot[w - 1] : 0);
        if (i < nblocks) block_sum[i] = excl;
        __syncthreads();  // every thread has read carry and warp_tot
        if (threadIdx.x == 1023) carry = excl + n;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

constexpr int kMeshWarps = 2;  // shared memory: 2 x (15 x 344 mass-property terms + 241 vertices)

__global__ void __launch_bounds__(kMeshWarps * 32) k_mesh(PrepArgs a) {
    __shared__ float s_g[kMeshWarps][kGenomeN + 1];
    __shared__ vec3 s_v[kMeshWarps][kNvMax];
    __shared__ float s_com[kMeshWarps][4];
    __shared__ float s_terms[kMeshWarps][kMpTerms * kNtMax];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int p = blockIdx.x * kMeshWarps + w;
    if (p >= a.pop) return;  // warp-uniform; no block barrier follows
    const float* src = a.genomes + (size_t)p * kGenomeN;
    for (int i = lane; i < kGenomeN; i += 32) s_g[w][i] = src[i];
    __syncwarp();
    GenomeRef g{s_g[w]};
    const Topo tp = topology(g);
    for (int i = lane; i < tp.nv; i += 32) s_v[w][i] = mesh_vertex(g, tp, i);
    __syncwarp();

    // mesh extent (min/max are exact in any order), src/common.h:294-307
    vec3 lo = s_v[w][0], hi = lo;
    for (int i = lane; i < tp.nv; i += 32) {
        vec3 v = s_v[w][i];
        lo.x = fminf(lo.x, v.x); lo.y = fminf(lo.y, v.y); lo.z = fminf(lo.z, v.z);
        hi.x = fmaxf(hi.x, v.x); hi.y = fmaxf(hi.y, v.y); hi.z = fmaxf(hi.z, v.z);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo.x = fminf(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
        lo.y = fminf(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
        lo.z = fminf(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
        hi.x = fmaxf(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
        hi.y = fmaxf(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
        hi.z = fmaxf(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
    }
    vec3 ext = vsub(hi, lo);
    const float lim = PE_PRINT_LIMIT;
    const int printable = ext.x <= lim && ext.y <= lim && ext.z <= lim;
    const int nt = printable ? tp.nt : 0;
    const int off = a.pt.off[p] + a.block_sum[p / kScanBlock];

    MassProps mp;
    mass_props(g, s_v[w], tp, lane, s_terms[w], s_com[w], &mp);
    if (lane == 0) {
        float* o = a.pt.mp + (size_t)p * kMpN;
        o[0] = mp.mass; o[1] = mp.invmass; o[2] = mp.com.x; o[3] = mp.com.y; o[4] = mp.com.z;
        for (int k = 0; k < 6; k++) o[5 + k] = mp.I[k];
        for (int k = 0; k < 9; k++) o[11 + k] = mp.invI[k];
        s_com[w][0] = mp.com.x; s_com[w][1] = mp.com.y; s_com[w][2] = mp.com.z;
        a.pt.nt[p] = nt;
        a.pt.ext[p] = make_float4(ext.x, ext.y, ext.z, (float)tp.nt);
    }
    __syncwarp();
    if (lane == 0) a.pt.off[p] = off;
    const vec3 com = mk3(s_com[w][0], s_com[w][1], s_com[w][2]);
    // COM-relative panels, src/sim.cu:40-48
    for (int t = lane; t < nt; t += 32) {
        int ia, ib, ic; mesh_tri(tp, t, &ia, &ib, &ic);
        vec3 pa = vsub(s_v[w][ia], com), pb = vsub(s_v[w][ib], com), pcv = vsub(s_v[w][ic], com);
        vec3 nrm = vcross(vsub(pb, pa), vsub(pcv, pa));
        float A = 0.5f * vlen(nrm);
        vec3 ct = vscl(vadd(vadd(pa, pb), pcv), 1.0f / 3);
        a.pc[off + t] = make_float4(ct.x, ct.y, ct.z, A);
        vec3 n = A > 1e-12f ? vscl(nrm, 0.5f / A) : mk3(0, 0, 1);
        a.pn[off + t] = make_float4(n.x, n.y, n.z, 0.0f);
    }
}

cudaError_t set_station_mode(int ieee) {
    int v = ieee ? 1 : 0;
    return cudaMemcpyToSymbol(c_station_ieee, &v, sizeof(int));
}

void launch_prepare(const PrepArgs& a, int* d_total, cudaStream_t s) {
    int nb = (a.pop + kScanBlock - 1) / kScanBlock;
    k_topo_scan<<<nb, kScanBlock, 0, s>>>(a);
    k_scan_tot<<<1, 1024, 0, s>>>(a.block_sum, nb, d_total);
    k_mesh<<<(a.pop + kMeshWarps - 1) / kMeshWarps, kMeshWarps * 32, 0, s>>>(a);
}

}  // namespace pe
