// pe_grad.cu -- d(objective)/d(genome) on the GPU: the reverse-mode flight adjoint with
// trajectory checkpoints and segment recompute, and the forward-mode genome contraction.
//
// The objective of a genome is the tail-aware score (0.65 mean + 0.25 mean of the worst
// ceil(S/4) + 0.10 worst, src/sim.cu:340-357) of its smoothed landing distances (the z = 0
// crossing interpolated between the last two states; src/sim.cu:198-204 ends the flight there).
// The model and its adjoint are the templates of pe_grad_model.h, instantiated in float here;
// this file is built without fast math so the gust sines (arguments up to ~100 rad) and the
// divisions stay IEEE.
//
// Pipeline on one stream, after prepare (pe_prepare.cu) has written the plane table and panels:
//   k_grad_setup    thread per flight: this model's print variation, scenario and release, as a
//                   record for the forward pass.
//   forward         the evaluation's body-frame flight kernel (pe_flight_fast.cu, its GRAD
//                   instance) on those records: packed f32x2 panel pairs, smoothed distance, step
//                   count, how the flight ended, the state every K steps and every step's
//                   body-frame force and torque.
//   k_grad_order    one block: flights sorted by step count, longest first (counting sort), so
//                   the reverse pass starts its longest flights first.
//   k_grad_reverse  a block of W warps per flight in that order: per segment of K steps (last
//                   first) the states are rebuilt from the checkpoint through this model's
//                   integrator on the forward's stored forces (or, when those were not kept, its
//                   panel pass too) into shared memory, then the adjoint runs back over the
//                   segment.  The rebuilt states differ from the forward's by the rounding of two
//                   float implementations of one step over at most K steps; the adjoint is taken
//                   along them.  Each thread owns the adjoint accumulators of its panels.  Writes
//                   the adjoint of the plane data (mass, inertia, panel centroids, areas and
//                   normals) per flight.
//   k_grad_weights  one block per plane: tail weights of its distances and the weighted sum of its
//                   flights' adjoints (ybar).
//   k_grad_genome   one block per (plane, gene): a dual-number pass with that gene's tangent
//                   through mesh -> mass_props -> panels, parallel over vertices and triangles,
//                   dotted with ybar.
#include <cuda_runtime.h>

#include <cstddef>

#include "pe_f32x2.cuh"
#include "pe_grad_model.h"
#include "pe_internal.cuh"

#ifndef GRAD_REV_WARPS
#define GRAD_REV_WARPS 4
#endif
#ifndef GRAD_SOLO
#define GRAD_SOLO 1
#endif
#ifndef GRAD_REV_GROUP
#define GRAD_REV_GROUP 2
#endif
#ifndef GRAD_GROUP_WARPS
#define GRAD_GROUP_WARPS 3
#endif

namespace pe {

namespace {

using F3 = pg::V3<float>;
using FSt = pg::St<float>;

constexpr int kPanelFloats = 7 * kNtMax;  // rbx rby rbz nbx nby nbz ak (SoA)
constexpr int kSegFloats = 20;            // state (14) + body force (3) + body torque (3)
constexpr int kCkFloats = 16;             // one checkpointed state

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ FSt zero_state() {
    FSt z;
    z.pos = pg::v3(0.f, 0.f, 0.f);
    z.vel = z.pos;
    z.w = z.pos;
    z.q[0] = z.q[1] = z.q[2] = z.q[3] = 0.f;
    z.t = 0.f;
    return z;
}

// Constants of one flight: scenario draw, print variation, gust phase.
struct FlightCtx {
    pg::FlightP<float> P;
    F3 cg;
    float sigma, beta[6];
    float sc[kScenN];
    int nt, off;
};

__device__ __forceinline__ void flight_setup(const GradArgs& a, int f, FlightCtx& c) {
    const int p = f / a.nseeds, s = f - p * a.nseeds;
    const int seed = a.seeds[s] + (a.vary ? p * 7919 : 0);
    Scenario S;
    scenario_desc(seed, &S);
#pragma unroll
    for (int k = 0; k < kScenN; k++) c.sc[k] = S.v[k];
    const float* mp = a.plane_mp + (size_t)p * kMpN;
    float I[6];
#pragma unroll
    for (int k = 0; k < 6; k++) I[k] = mp[5 + k];
    pg::printed(c.sc, mp[0], I, c.P, &c.cg, &c.sigma, c.beta);
    c.P.phase = seed_phase(seed);
    c.nt = a.plane_nt[p];
    c.off = a.plane_off[p];
}

// A flight's constants as k_grad_setup wrote them: the forward pass flew with these, and every
// reverse kernel takes them from here rather than from its own flight_setup, whose rounding may
// differ in the last place with how the compiler fuses it into each kernel.
__device__ __forceinline__ pg::FlightP<float> setup_flightp(const GradArgs& a, int f) {
    const float* r = a.setup + (size_t)f * kGradSetupFloats;
    pg::FlightP<float> P;
    P.mass = r[0];
    P.invmass = r[1];
#pragma unroll
    for (int k = 0; k < 6; k++) P.I[k] = r[2 + k];
#pragma unroll
    for (int k = 0; k < 9; k++) P.invI[k] = r[8 + k];
    P.cf = r[17];
    P.phase = r[18];
    P.gust = r[19];
    P.base_x = r[20];
    P.base_y = r[21];
    return P;
}

// Print-warped body-frame panels of one flight into shared memory (SoA), by all nthr threads.
__device__ __forceinline__ void stage_panels(const GradArgs& a, const FlightCtx& c, float* sp, int tid, int nthr) {
    if ((c.nt & 1) && tid < 7) sp[tid * kNtMax + c.nt] = 0.f;  // an odd plane's last pair: a zero panel
    for (int i = tid; i < c.nt; i += nthr) {
        const float4 c4 = a.pc[c.off + i], n4 = a.pn[c.off + i];
        F3 rb, nb;
        float ak;
        pg::stage(pg::v3(c4.x, c4.y, c4.z), c4.w, pg::v3(n4.x, n4.y, n4.z), c.cg, c.sc[pg::SC_RHO], c.sc[pg::SC_WP],
                  c.sc[pg::SC_WR], &rb, &nb, &ak);
        sp[0 * kNtMax + i] = rb.x; sp[1 * kNtMax + i] = rb.y; sp[2 * kNtMax + i] = rb.z;
        sp[3 * kNtMax + i] = nb.x; sp[4 * kNtMax + i] = nb.y; sp[5 * kNtMax + i] = nb.z;
        sp[6 * kNtMax + i] = ak;
    }
}

// This thread's share of the body-frame force and torque, summed over its warp (every lane gets
// it).  Panels i = tid, tid + nthr, ... -- at most PPT of them, all unrolled so their dependent
// chains (~300 cycles each) overlap instead of running one after another.
template <int PPT>
__device__ __forceinline__ void panel_partial(const pg::Pre<float>& pr, const float* sp, int nt, float cf, int tid,
                                              int nthr, float out[6]) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, a4 = 0.f, a5 = 0.f;
#pragma unroll
    for (int k = 0; k < PPT; k++) {  // branch-free: a slot past nt evaluates panel 0 and adds nothing
        const int i0 = tid + k * nthr;
        const bool on = i0 < nt;
        const int i = on ? i0 : 0;
        F3 rb = pg::v3(sp[i], sp[kNtMax + i], sp[2 * kNtMax + i]);
        F3 nb = pg::v3(sp[3 * kNtMax + i], sp[4 * kNtMax + i], sp[5 * kNtMax + i]);
        F3 f, tq;
        pg::panel_fwd(pr, rb, nb, sp[6 * kNtMax + i], cf, &f, &tq);
        a0 += on ? f.x : 0.f; a1 += on ? f.y : 0.f; a2 += on ? f.z : 0.f;
        a3 += on ? tq.x : 0.f; a4 += on ? tq.y : 0.f; a5 += on ? tq.z : 0.f;
    }
    out[0] = warp_sum(a0); out[1] = warp_sum(a1); out[2] = warp_sum(a2);
    out[3] = warp_sum(a3); out[4] = warp_sum(a4); out[5] = warp_sum(a5);
}

// panel_partial over the slots this flight fills: a block's threads all fly one plane, so the
// branch is uniform, and a plane of at most (PPT - 1) * nthr panels skips the last slot, which
// could only add +0.
template <int W>
__device__ __forceinline__ void panel_partial_nt(const pg::Pre<float>& pr, const float* sp, int nt, float cf, int tid,
                                                 float out[6]) {
    constexpr int nthr = 32 * W, PPT = (kNtMax + nthr - 1) / nthr;
    if (PPT > 1 && nt <= (PPT - 1) * nthr) panel_partial<(PPT > 1 ? PPT - 1 : 1)>(pr, sp, nt, cf, tid, nthr, out);
    else panel_partial<PPT>(pr, sp, nt, cf, tid, nthr, out);
}

__device__ __forceinline__ void store_state16(float* dst, const FSt& s) {
    float4* d4 = reinterpret_cast<float4*>(dst);
    d4[0] = make_float4(s.pos.x, s.pos.y, s.pos.z, s.q[0]);
    d4[1] = make_float4(s.q[1], s.q[2], s.q[3], s.vel.x);
    d4[2] = make_float4(s.vel.y, s.vel.z, s.w.x, s.w.y);
    d4[3] = make_float4(s.w.z, s.t, 0.f, 0.f);
}
__device__ __forceinline__ FSt load_state16(const float* src) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    const float4 a = s4[0], b = s4[1], c = s4[2], d = s4[3];
    FSt s;
    s.pos = pg::v3(a.x, a.y, a.z);
    s.q[0] = a.w; s.q[1] = b.x; s.q[2] = b.y; s.q[3] = b.z;
    s.vel = pg::v3(b.w, c.x, c.y);
    s.w = pg::v3(c.z, c.w, d.x);
    s.t = d.y;
    return s;
}
// A step's body force and torque as the forward pass stores them (2 float4).
__device__ __forceinline__ void store_fsum(float* dst, F3 F, F3 T) {
    float4* d4 = reinterpret_cast<float4*>(dst);
    d4[0] = make_float4(F.x, F.y, F.z, T.x);
    d4[1] = make_float4(T.y, T.z, 0.f, 0.f);
}
__device__ __forceinline__ void load_fsum(const float* src, F3* F, F3* T) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    const float4 a = s4[0], b = s4[1];
    *F = pg::v3(a.x, a.y, a.z);
    *T = pg::v3(a.w, b.x, b.y);
}
// Segment entry: the state before a step and that step's body force and torque (5 float4).
__device__ __forceinline__ void store_seg(float* dst, const FSt& s, F3 F, F3 T) {
    float4* d4 = reinterpret_cast<float4*>(dst);
    d4[0] = make_float4(s.pos.x, s.pos.y, s.pos.z, s.q[0]);
    d4[1] = make_float4(s.q[1], s.q[2], s.q[3], s.vel.x);
    d4[2] = make_float4(s.vel.y, s.vel.z, s.w.x, s.w.y);
    d4[3] = make_float4(s.w.z, s.t, F.x, F.y);
    d4[4] = make_float4(F.z, T.x, T.y, T.z);
}
__device__ __forceinline__ FSt load_seg(const float* src, F3* F, F3* T) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    const float4 a = s4[0], b = s4[1], c = s4[2], d = s4[3], e = s4[4];
    FSt s;
    s.pos = pg::v3(a.x, a.y, a.z);
    s.q[0] = a.w; s.q[1] = b.x; s.q[2] = b.y; s.q[3] = b.z;
    s.vel = pg::v3(b.w, c.x, c.y);
    s.w = pg::v3(c.z, c.w, d.x);
    s.t = d.y;
    *F = pg::v3(d.z, d.w, e.x);
    *T = pg::v3(e.y, e.z, e.w);
    return s;
}

// A rebuilt step of the pipelined reverse pass (kEntFloats): the state before the step and what
// the step's adjoint reads -- the body force and torque, the step's (va, vb) and gust Jacobian
// (step_pre), and the integrator's intermediates (step_post_f):
//   [0..13] pos q vel w t  [14..16] Fb  [17..19] Tb  [20..22] va  [23..25] vb  [26..34] J
//   [35..37] Fw  [38..40] Iw  [41..43] tq  [44..46] w1  [47..49] wn  [50..52] vel1  [53..56] qo  [57] il
constexpr int kEntFloats = 60;

__device__ __forceinline__ void put3(float* d, F3 v) { d[0] = v.x; d[1] = v.y; d[2] = v.z; }
__device__ __forceinline__ F3 get3(const float* d) { return pg::v3(d[0], d[1], d[2]); }

// The integrator's part of an entry (state, forces, intermediates), written by one lane.
__device__ __forceinline__ void put_entry_post(float* e, const FSt& s, F3 Fb, F3 Tb, const pg::PostF<float>& f) {
    put3(e, s.pos);
    e[3] = s.q[0]; e[4] = s.q[1]; e[5] = s.q[2]; e[6] = s.q[3];
    put3(e + 7, s.vel); put3(e + 10, s.w); e[13] = s.t;
    put3(e + 14, Fb); put3(e + 17, Tb);
    put3(e + 35, f.Fw); put3(e + 38, f.Iw); put3(e + 41, f.tq); put3(e + 44, f.w1); put3(e + 47, f.wn);
    put3(e + 50, f.vel1);
    e[53] = f.qo[0]; e[54] = f.qo[1]; e[55] = f.qo[2]; e[56] = f.qo[3]; e[57] = f.il;
}
__device__ __forceinline__ FSt get_entry_state(const float* e) {
    FSt s;
    s.pos = get3(e);
    s.q[0] = e[3]; s.q[1] = e[4]; s.q[2] = e[5]; s.q[3] = e[6];
    s.vel = get3(e + 7); s.w = get3(e + 10); s.t = e[13];
    return s;
}

// Per-block exchange area: each warp's partial sums for the current step (double-buffered by step
// parity, so one barrier per step suffices when every warp integrates); when only warp 0
// integrates, the (vb, w) it publishes for the panel pass, the flight's end flag and, in the
// reverse pass, (LFb, LTb); the flight index of the work queue.
template <int W>
struct StepShared {
    float part[2][W][8];  // [parity][warp] 6 partial sums
    float pre[8];         // vb xyz, w xyz, end flag
    float adj[8];         // LFb xyz, LTb xyz
    float after[16];      // reverse pass: the state after a flight's last step (from warp 0 or 1)
    float rcur[16];       // pipelined reverse pass: warp 1's rebuilt state between steps
    int rchunk;           // and its steps to the next 600-step clock restart
    int flight;
    int pad[2];
};
__device__ __forceinline__ void publish(float* pre, const pg::Pre<float>& pr, float done) {
    pre[0] = pr.vb.x; pre[1] = pr.vb.y; pre[2] = pr.vb.z;
    pre[3] = pr.w.x; pre[4] = pr.w.y; pre[5] = pr.w.z;
    pre[6] = done;
}
__device__ __forceinline__ void subscribe(const float* pre, pg::Pre<float>& pr) {
    pr.vb = pg::v3(pre[0], pre[1], pre[2]);
    pr.w = pg::v3(pre[3], pre[4], pre[5]);
}
template <int W>
__host__ __device__ constexpr int shared_head_floats() { return (int)((sizeof(StepShared<W>) + 15) / 16 * 4); }
using StepShared4 = StepShared<4>;
static_assert(offsetof(StepShared4, after) % 16 == 0 && offsetof(StepShared4, rcur) % 16 == 0,
              "states are stored and loaded as float4");

// Sum of the warps' partials in warp order (every warp gets bit-identical totals).
template <int W>
__device__ __forceinline__ void sum_parts(const float (*part)[8], F3* A, F3* B) {
    float v[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        float t = part[0][k];
#pragma unroll
        for (int w = 1; w < W; w++) t += part[w][k];
        v[k] = t;
    }
    *A = pg::v3(v[0], v[1], v[2]);
    *B = pg::v3(v[3], v[4], v[5]);
}
__device__ __forceinline__ void put_part(float* dst, const float v[6]) {
#pragma unroll
    for (int k = 0; k < 6; k++) dst[k] = v[k];
}

template <int W>
__device__ __forceinline__ int block_next_flight(StepShared<W>& sh, int* counter) {
    if (threadIdx.x == 0) sh.flight = atomicAdd(counter, 1);
    __syncthreads();
    const int f = sh.flight;
    __syncthreads();
    return f;
}

// ------------------------------------------------------------------ set-up of the forward pass
// Each flight's constants (print variation, scenario, gust field) and release state from this
// model, written as the record the forward pass reads (kGradSetupFloats): the forward then flies
// the flight the reverse pass differentiates, whatever the scenario seed.
__global__ void __launch_bounds__(128) k_grad_setup(GradArgs a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.n_flights) return;
    FlightCtx c;
    flight_setup(a, f, c);
    float* r = a.setup + (size_t)f * kGradSetupFloats;
    r[0] = c.P.mass; r[1] = c.P.invmass;
#pragma unroll
    for (int k = 0; k < 6; k++) r[2 + k] = c.P.I[k];
#pragma unroll
    for (int k = 0; k < 9; k++) r[8 + k] = c.P.invI[k];
    r[17] = c.P.cf; r[18] = c.P.phase; r[19] = c.P.gust; r[20] = c.P.base_x; r[21] = c.P.base_y;
    r[22] = c.cg.x; r[23] = c.cg.y; r[24] = c.cg.z;
    r[25] = c.sc[pg::SC_RHO]; r[26] = c.sc[pg::SC_WP]; r[27] = c.sc[pg::SC_WR];
    r[28] = r[29] = r[30] = r[31] = 0.f;
    const FSt s = pg::release(c.sc, c.P, c.cg, (F3*)nullptr, (F3*)nullptr);
    store_state16(r + 32, s);  // pos, q, vel, w, t (FlightState layout); step 0
    r[46] = 0.f;
    r[47] = 0.f;
}

// ------------------------------------------------------------------ longest flights first
constexpr int kOrderThreads = 1024;
__global__ void __launch_bounds__(kOrderThreads) k_grad_order(const int* steps, int n, int* order) {
    __shared__ int hist[kMaxSteps + 1];
    __shared__ int warp_tot[kOrderThreads / 32];
    const int tid = threadIdx.x;
    for (int b = tid; b <= kMaxSteps; b += kOrderThreads) hist[b] = 0;
    __syncthreads();
    for (int f = tid; f < n; f += kOrderThreads) atomicAdd(&hist[kMaxSteps - steps[f]], 1);
    __syncthreads();
    // exclusive scan of hist: each thread owns a contiguous run of bins
    constexpr int kPer = (kMaxSteps + 1 + kOrderThreads - 1) / kOrderThreads;
    const int b0 = tid * kPer;
    int run = 0;
    for (int b = b0; b < b0 + kPer && b <= kMaxSteps; b++) run += hist[b];
    int incl = run;
    const int lane = tid & 31, w = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = warp_tot[lane];
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        warp_tot[lane] = x - v;
    }
    __syncthreads();
    int base = warp_tot[w] + incl - run;
    for (int b = b0; b < b0 + kPer && b <= kMaxSteps; b++) {
        const int h = hist[b];
        hist[b] = base;
        base += h;
    }
    __syncthreads();
    for (int f = tid; f < n; f += kOrderThreads) order[atomicAdd(&hist[kMaxSteps - steps[f]], 1)] = f;
}

// ------------------------------------------------------------------ reverse sweep
// Per-step constants of the packed panel adjoint (both halves equal).
struct AdjK {
    f2 vbx, vby, vbz, wx, wy, wz, nwx, nwy, nwz;  // body air velocity, body rates and their negation
    f2 nLFx, nLFy, nLFz, LTx, LTy, LTz, nLTx, nLTy, nLTz;  // -LFb, LTb, -LTb
    f2 cf, k19, tiny, mone, m05;
};
__device__ __forceinline__ AdjK adj_consts(const pg::Pre<float>& pr, float cf, F3 LFb, F3 LTb) {
    AdjK k;
    k.vbx = bc(pr.vb.x); k.vby = bc(pr.vb.y); k.vbz = bc(pr.vb.z);
    k.wx = bc(pr.w.x); k.wy = bc(pr.w.y); k.wz = bc(pr.w.z);
    k.nwx = bc(-pr.w.x); k.nwy = bc(-pr.w.y); k.nwz = bc(-pr.w.z);
    k.nLFx = bc(-LFb.x); k.nLFy = bc(-LFb.y); k.nLFz = bc(-LFb.z);
    k.LTx = bc(LTb.x); k.LTy = bc(LTb.y); k.LTz = bc(LTb.z);
    k.nLTx = bc(-LTb.x); k.nLTy = bc(-LTb.y); k.nLTz = bc(-LTb.z);
    k.cf = bc(cf); k.k19 = bc(1.9f); k.tiny = bc(1e-30f); k.mone = bc(-1.f); k.m05 = bc(-0.5f);
    return k;
}

// Packed partial sums of a thread's share of the step's (Lvb, Lw): even panels low, odd high.
struct AdjAcc {
    f2 vx, vy, vz, wx, wy, wz;
};

// The adjoint of the panel force (panel_fwd of the model) for the two panels of pair q, two panels
// per f32x2 instruction: accumulates the panels' own adjoints (Lrb, Lnb, Lak) in place in sa and
// adds their shares of (Lvb, Lw) to acc.  A panel below 1 mm/s of relative flow is not skipped: the
// 1e-30 added to |vr|^2 keeps 1/|vr| finite and its contributions vanish with its force, as in the
// forward pass.  A zero panel (the pad of an odd plane) contributes exact zeros.
__device__ __forceinline__ void adj_pair(const AdjK& k, const float* sp, float* sa, int q, bool on, AdjAcc& acc) {
    const float2* s2 = reinterpret_cast<const float2*>(sp);
    float2* a2 = reinterpret_cast<float2*>(sa);
    constexpr int P2 = kNtMax / 2;  // pairs per field
    const float2 Rx = s2[q], Ry = s2[P2 + q], Rz = s2[2 * P2 + q];
    const float2 Nx = s2[3 * P2 + q], Ny = s2[4 * P2 + q], Nz = s2[5 * P2 + q], Ak = s2[6 * P2 + q];
    const f2 rbx = pk(Rx.x, Rx.y), rby = pk(Ry.x, Ry.y), rbz = pk(Rz.x, Rz.y);
    const f2 nbx = pk(Nx.x, Nx.y), nby = pk(Ny.x, Ny.y), nbz = pk(Nz.x, Nz.y), ak = pk(Ak.x, Ak.y);
    // forward quantities: vr = vb + w x rb, |vr|^2, 1/|vr|, s, qd, sqrt(1 - s^2), gf, na, nv, -f
    const f2 vrx = fma2(k.wy, rbz, fma2(k.nwz, rby, k.vbx));
    const f2 vry = fma2(k.wz, rbx, fma2(k.nwx, rbz, k.vby));
    const f2 vrz = fma2(k.wx, rby, fma2(k.nwy, rbx, k.vbz));
    const f2 V2 = fma2(vrz, vrz, fma2(vry, vry, fma2(vrx, vrx, k.tiny)));
    float v2a, v2b;
    upk(V2, v2a, v2b);
    const f2 inv = pk(pg::p_rsqrt(v2a), pg::p_rsqrt(v2b));
    const f2 vn = fma2(vrz, nbz, fma2(vry, nby, mul2(vrx, nbx)));
    const f2 s = mul2(vn, inv);
    const f2 qd = mul2(V2, ak);
    float sa_, sb_, ua, ub;
    upk(s, sa_, sb_);
    upk(fma2(s, s, k.mone), ua, ub);  // s^2 - 1
    ua = -ua;
    ub = -ub;
    const float sqa = pg::p_sqrt_nn(fmaxf(0.f, ua)), sqb = pg::p_sqrt_nn(fmaxf(0.f, ub));
    const f2 sq = pk(sqa, sqb);
    float cfs, cfs2;
    upk(k.cf, cfs, cfs2);
    const f2 gf = fma2(k.k19, sq, pk(fmaf(2.f, fabsf(sa_), -cfs), fmaf(2.f, fabsf(sb_), -cfs)));
    const f2 na = mul2(mul2(qd, s), gf);
    const f2 nv = mul2(mul2(qd, k.cf), inv);
    const f2 nfx = fma2(na, nbx, mul2(nv, vrx));  // -f
    const f2 nfy = fma2(na, nby, mul2(nv, vry));
    const f2 nfz = fma2(na, nbz, mul2(nv, vrz));
    // adjoint: Lnf = -(LF + LT x rb) = -LF + rb x LT
    const f2 Lnfx = fma2(rby, k.LTz, fma2(rbz, k.nLTy, k.nLFx));
    const f2 Lnfy = fma2(rbz, k.LTx, fma2(rbx, k.nLTz, k.nLFy));
    const f2 Lnfz = fma2(rbx, k.LTy, fma2(rby, k.nLTx, k.nLFz));
    float2 Lrx = a2[q], Lry = a2[P2 + q], Lrz = a2[2 * P2 + q];
    float2 Lnx = a2[3 * P2 + q], Lny = a2[4 * P2 + q], Lnz = a2[5 * P2 + q], Lak2 = a2[6 * P2 + q];
    f2 Lrbx = pk(Lrx.x, Lrx.y), Lrby = pk(Lry.x, Lry.y), Lrbz = pk(Lrz.x, Lrz.y);
    f2 Lnbx = pk(Lnx.x, Lnx.y), Lnby = pk(Lny.x, Lny.y), Lnbz = pk(Lnz.x, Lnz.y), Lak = pk(Lak2.x, Lak2.y);
    // Lrb += f x LT = LT x (-f)
    Lrbx = fma2(k.LTy, nfz, fma2(k.nLTz, nfy, Lrbx));
    Lrby = fma2(k.LTz, nfx, fma2(k.nLTx, nfz, Lrby));
    Lrbz = fma2(k.LTx, nfy, fma2(k.nLTy, nfx, Lrbz));
    const f2 Lna = fma2(Lnfz, nbz, fma2(Lnfy, nby, mul2(Lnfx, nbx)));
    Lnbx = fma2(Lnfx, na, Lnbx);
    Lnby = fma2(Lnfy, na, Lnby);
    Lnbz = fma2(Lnfz, na, Lnbz);
    const f2 Lnv = fma2(Lnfz, vrz, fma2(Lnfy, vry, mul2(Lnfx, vrx)));
    f2 Lvrx = mul2(Lnfx, nv), Lvry = mul2(Lnfy, nv), Lvrz = mul2(Lnfz, nv);
    const f2 Lqd = fma2(mul2(Lnv, k.cf), inv, mul2(mul2(Lna, s), gf));
    f2 Linv = mul2(mul2(Lnv, qd), k.cf);
    const f2 Lgf = mul2(mul2(Lna, qd), s);
    float lsa, lsb, lga, lgb;
    upk(mul2(Lna, mul2(qd, gf)), lsa, lsb);
    upk(Lgf, lga, lgb);
    // d gf / d s = 2 sign(s) + 1.9 d sqrt(1 - s^2) / d s
    lsa = fmaf(sa_ < 0.f ? -2.f : 2.f, lga, lsa);
    lsb = fmaf(sb_ < 0.f ? -2.f : 2.f, lgb, lsb);
    if (ua > 0.f && sqa > 1e-6f) lsa -= 1.9f * lga * sa_ * pg::p_rcp(sqa);
    if (ub > 0.f && sqb > 1e-6f) lsb -= 1.9f * lgb * sb_ * pg::p_rcp(sqb);
    const f2 Ls = pk(lsa, lsb);
    f2 LV2 = mul2(Lqd, ak);
    Lak = fma2(Lqd, V2, Lak);
    const f2 Lvn = mul2(Ls, inv);
    Linv = fma2(Ls, vn, Linv);
    Lvrx = fma2(nbx, Lvn, Lvrx);
    Lvry = fma2(nby, Lvn, Lvry);
    Lvrz = fma2(nbz, Lvn, Lvrz);
    Lnbx = fma2(vrx, Lvn, Lnbx);
    Lnby = fma2(vry, Lvn, Lnby);
    Lnbz = fma2(vrz, Lvn, Lnbz);
    LV2 = fma2(Linv, mul2(k.m05, mul2(inv, mul2(inv, inv))), LV2);
    const f2 LV22 = add2(LV2, LV2);
    Lvrx = fma2(vrx, LV22, Lvrx);
    Lvry = fma2(vry, LV22, Lvry);
    Lvrz = fma2(vrz, LV22, Lvrz);
    // Lrb += Lvr x w
    Lrbx = fma2(Lvry, k.wz, fma2(Lvrz, k.nwy, Lrbx));
    Lrby = fma2(Lvrz, k.wx, fma2(Lvrx, k.nwz, Lrby));
    Lrbz = fma2(Lvrx, k.wy, fma2(Lvry, k.nwx, Lrbz));
    if (on) {  // a slot past the plane's pairs evaluated pair 0 and keeps nothing
        float2 o;
        upk(Lrbx, o.x, o.y); a2[q] = o;
        upk(Lrby, o.x, o.y); a2[P2 + q] = o;
        upk(Lrbz, o.x, o.y); a2[2 * P2 + q] = o;
        upk(Lnbx, o.x, o.y); a2[3 * P2 + q] = o;
        upk(Lnby, o.x, o.y); a2[4 * P2 + q] = o;
        upk(Lnbz, o.x, o.y); a2[5 * P2 + q] = o;
        upk(Lak, o.x, o.y); a2[6 * P2 + q] = o;
        // Lvb += Lvr;  Lw += rb x Lvr
        acc.vx = add2(acc.vx, Lvrx);
        acc.vy = add2(acc.vy, Lvry);
        acc.vz = add2(acc.vz, Lvrz);
        acc.wx = sub2(fma2(rby, Lvrz, acc.wx), mul2(rbz, Lvry));
        acc.wy = sub2(fma2(rbz, Lvrx, acc.wy), mul2(rbx, Lvrz));
        acc.wz = sub2(fma2(rbx, Lvry, acc.wz), mul2(rby, Lvrx));
    }
}

// The panel adjoint of one step: this thread's pairs (at most PP of them, all unrolled so their
// chains overlap); the (Lvb, Lw) shares summed over them, then low + high.  Slot c holds pairs
// c nthr .. (c + 1) nthr - 1; even slots run up the threads, odd slots down, so a plane's last
// partial slot falls on the highest warps, away from warp 0 and its integrator.  A warp with no
// pair in a slot skips it.
template <int PP>
__device__ __forceinline__ void adj_panels(const pg::Pre<float>& pr, const float* sp, float* sa, int nt, float cf,
                                           F3 LFb, F3 LTb, int tid, int nthr, F3* Lvb_out, F3* Lwp_out) {
    const AdjK k = adj_consts(pr, cf, LFb, LTb);
    const int npairs = (nt + 1) >> 1;
    AdjAcc acc;
    acc.vx = acc.vy = acc.vz = acc.wx = acc.wy = acc.wz = 0ull;
    const int wbase = tid & ~31;
#pragma unroll
    for (int c = 0; c < PP; c++) {
        const int q0 = c * nthr + ((c & 1) ? nthr - 1 - tid : tid);
        // the lowest pair a lane of this warp holds in slot c: uniform over the warp
        const int qw = c * nthr + ((c & 1) ? nthr - 32 - wbase : wbase);
        if (qw >= npairs) continue;
        const bool on = q0 < npairs;
        adj_pair(k, sp, sa, on ? q0 : 0, on, acc);
    }
    float lo, hi;
    F3 v, w;
    upk(acc.vx, lo, hi); v.x = lo + hi;
    upk(acc.vy, lo, hi); v.y = lo + hi;
    upk(acc.vz, lo, hi); v.z = lo + hi;
    upk(acc.wx, lo, hi); w.x = lo + hi;
    upk(acc.wy, lo, hi); w.y = lo + hi;
    upk(acc.wz, lo, hi); w.z = lo + hi;
    *Lvb_out = v;
    *Lwp_out = w;
}

// One block of W warps per flight, flights in the order k_grad_order wrote.  Per segment of K
// steps (last first): rebuild the states from the checkpoint into shared memory, then the adjoint
// step by step.  Each thread accumulates its panels' adjoints in shared memory and its share of
// (Lvb, Lw), which the warps exchange.  SOLO = false: the integrator's adjoint runs in every warp
// from the same totals (one barrier per step); SOLO = true: in warp 0, which publishes
// (vb, w, LFb, LTb) for the panel pass (two barriers per step).
// LONG = true: the pipelined pass for the longest flights, one flight per block (order indices
// 0 .. n_long - 1), at the register count the pipeline needs.  While warp 0 differentiates segment
// sg step by step and every warp runs the panel adjoint, warp 1 rebuilds segment sg - 1 from its
// checkpoint and the stored forces, one step per step, keeping the integrator's intermediates, and
// warp 2 evaluates each rebuilt step's step_pre and gust Jacobian one step behind; warp 0's chain
// holds only the adjoint arithmetic.  Needs SOLO, W >= 3, stored forces and K <= kPipeMaxK.
// LONG = false: the other flights (order indices n_long ..), persistent over a work queue, at 3
// blocks per SM.
template <int W, bool SOLO, bool LONG>
__global__ void __launch_bounds__(32 * W, LONG ? 1 : (W >= 8 ? 1 : 12 / W)) k_grad_reverse(GradArgs a) {
    extern __shared__ __align__(16) float smem[];
    StepShared<W>& sh = *reinterpret_cast<StepShared<W>*>(smem);
    float* sp = smem + shared_head_floats<W>();  // staged panels
    float* sa = sp + kPanelFloats;                // per-panel adjoint accumulators (same layout)
    float* seg = sa + kPanelFloats;               // K entries of kSegFloats
    constexpr int nthr = 32 * W;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool scalar = !SOLO || warp == 0;
    // The longest flights' blocks are resident before the other flights' kernel starts: this kernel
    // lets its dependent launch begin at once, and that kernel waits for this one's completion
    // before it exits (programmatic dependent launch, below).
    if (LONG) asm volatile("griddepcontrol.launch_dependents;");
    for (int once = 0;; once++) {
        int idx;
        if (LONG) {
            if (once > 0) break;
            idx = blockIdx.x;
        } else {
            idx = a.n_long + block_next_flight(sh, &a.work[1]);
        }
        if (idx >= (LONG ? a.n_long : a.n_flights)) break;
        const int f = a.order[idx];
        float* out = a.adj + (size_t)f * kAdjStride;
        const int kind = a.kind[f];
        if (kind == 0 || kind == 3) {  // oversize or NaN flight: constant distance
            for (int i = tid; i < kAdjStride; i += nthr) out[i] = 0.f;
            continue;
        }
        pg::FlightP<float> P;
        int nt;
        {
            FlightCtx c;
            flight_setup(a, f, c);
            stage_panels(a, c, sp, tid, nthr);
            P = setup_flightp(a, f);
            nt = c.nt;
        }
        for (int i = tid; i < kPanelFloats; i += nthr) sa[i] = 0.f;
        const int k = a.steps[f] - 1;
        const float* ck = a.ck + (size_t)f * a.nck * kCkFloats;
        pg::LamP<float> LP;
        LP.mass = LP.invmass = 0.f;
#pragma unroll
        for (int q = 0; q < 6; q++) LP.I[q] = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) LP.invI[q] = 0.f;
        FSt Lnext = zero_state();
        F3 Lb_pos = pg::v3(0.f, 0.f, 0.f);
        int par = 0;
        if constexpr (LONG) {
            // the two segment buffers: segment g uses seg + (g & 1) * K entries
            auto ebuf = [&](int g) { return seg + (size_t)(g & 1) * a.K * kEntFloats; };
            const int S = k / a.K;
            const float* fs0 = a.fsum + (size_t)f * a.max_steps * 8;
            // warp 1: start rebuilding segment g from its checkpoint
            auto rebuild_start = [&](int g) {
                const FSt c0 = load_state16(ck + (size_t)g * kCkFloats);
                if (lane == 0) {
                    store_state16(sh.rcur, c0);
                    sh.rchunk = kChunk - (g * a.K) % kChunk;
                }
                __syncwarp();
            };
            // warp 1: the rebuilt steps n0..n1 - 1 of segment g into e, continuing from sh.rcur (the
            // state after the flight's last step into sh.after)
            auto rebuild = [&](int g, int n0, int n1, float* e) {
                const int j0g = g * a.K, j1g = min(j0g + a.K - 1, k);
                if (n0 >= n1 || j0g + n0 > j1g) return;
                FSt cur = load_state16(sh.rcur);
                int to_chunk = sh.rchunk;
                for (int n = n0; n < n1 && j0g + n <= j1g; n++) {
                    const int j = j0g + n;
                    pg::M3<float> R;
                    pg::rot_rows(cur.q, R);
                    F3 Fb, Tb;
                    load_fsum(fs0 + (size_t)j * 8, &Fb, &Tb);
                    pg::PostF<float> pf;
                    const FSt nx = pg::step_post_f(P, cur, R, Fb, Tb, pf);
                    if (lane == 0) put_entry_post(e + (size_t)n * kEntFloats, cur, Fb, Tb, pf);
                    if (j == k) {
                        if (lane == 0) store_state16(sh.after, nx);
                    } else {
                        cur = nx;
                        if (--to_chunk == 0) { cur.t = (float)(j + 1) * pg::kDt; to_chunk = kChunk; }  // src/sim.cu:113
                    }
                }
                __syncwarp();
                if (lane == 0) {
                    store_state16(sh.rcur, cur);
                    sh.rchunk = to_chunk;
                }
                __syncwarp();
            };
            // warp 2: step_pre and the gust Jacobian of the rebuilt steps n0..n1 - 1 of segment g
            auto pre = [&](int g, int n0, int n1, float* e) {
                const int len = min(g * a.K + a.K - 1, k) - g * a.K + 1;
                for (int n = n0; n < n1 && n < len; n++) {
                    float* en = e + (size_t)n * kEntFloats;
                    const FSt st = get_entry_state(en);
                    pg::Pre<float> q;
                    float J[3][3];
                    pg::step_pre(P, st, q, J);
                    if (lane == 0) {
                        put3(en + 20, q.va); put3(en + 23, q.vb);
#pragma unroll
                        for (int r = 0; r < 3; r++) put3(en + 26 + 3 * r, pg::v3(J[r][0], J[r][1], J[r][2]));
                    }
                }
            };
            // prologue: the flight's last segment, rebuilt before its adjoint starts
            if (warp == 1) {
                rebuild_start(S);
                rebuild(S, 0, a.K, ebuf(S));
            }
            __syncthreads();
            if (warp == 2) pre(S, 0, a.K, ebuf(S));
            __syncthreads();
            if (warp == 0) {
                const FSt before = get_entry_state(ebuf(S) + (size_t)(k - S * a.K) * kEntFloats);
                const FSt after = load_state16(sh.after);
                FSt Lb = zero_state();
                pg::terminate_adj(before, after, kind, Lb, Lnext);
                Lb_pos = Lb.pos;
            }
            for (int sg = S; sg >= 0; sg--) {
                const int j0 = sg * a.K, j1 = min(j0 + a.K - 1, k), len = j1 - j0 + 1;
                const float* ecur = ebuf(sg);
                float* enext = ebuf(sg + 1);  // segment sg - 1, rebuilt meanwhile
                if (warp == 1 && sg >= 1) rebuild_start(sg - 1);
                for (int n = 0; n < len; n++) {
                    const int j = j1 - n;
                    FSt st, L0;
                    pg::Pre<float> pr;
                    pg::M3<float> LR;
                    float J[3][3];
                    F3 LFb, LTb;
                    if (warp == 0) {
                        const float* e = ecur + (size_t)(j - j0) * kEntFloats;
                        st = get_entry_state(e);
                        const F3 Fb = get3(e + 14);
                        pr.va = get3(e + 20);
                        pr.vb = get3(e + 23);
                        pr.w = st.w;
#pragma unroll
                        for (int r = 0; r < 3; r++) { J[r][0] = e[26 + 3 * r]; J[r][1] = e[27 + 3 * r]; J[r][2] = e[28 + 3 * r]; }
                        pg::PostF<float> pf;
                        pf.Fw = get3(e + 35); pf.Iw = get3(e + 38); pf.tq = get3(e + 41); pf.w1 = get3(e + 44);
                        pf.wn = get3(e + 47); pf.vel1 = get3(e + 50);
                        pf.qo[0] = e[53]; pf.qo[1] = e[54]; pf.qo[2] = e[55]; pf.qo[3] = e[56]; pf.il = e[57];
                        pg::rot_rows(st.q, pr.R);
                        L0 = zero_state();
#pragma unroll
                        for (int r = 0; r < 3; r++)
#pragma unroll
                            for (int q = 0; q < 3; q++) LR.a[r][q] = 0.f;
                        pg::step_post_adj_f(P, st, pr.R, Fb, pf, Lnext, L0, &LFb, &LTb, LR, LP);
                        if (tid == 0) {
                            publish(sh.pre, pr, 0.f);
                            sh.adj[0] = LFb.x; sh.adj[1] = LFb.y; sh.adj[2] = LFb.z;
                            sh.adj[3] = LTb.x; sh.adj[4] = LTb.y; sh.adj[5] = LTb.z;
                        }
                    } else if (warp == 1 && sg >= 1) {
                        rebuild(sg - 1, n, n + 1, enext);
                    } else if (warp == 2 && sg >= 1 && n >= 1) {
                        pre(sg - 1, n - 1, n, enext);
                    }
                    __syncthreads();
                    subscribe(sh.pre, pr);
                    LFb = pg::v3(sh.adj[0], sh.adj[1], sh.adj[2]);
                    LTb = pg::v3(sh.adj[3], sh.adj[4], sh.adj[5]);
                    F3 Lvb, Lwp;
                    {
                        constexpr int PP = (kNtMax / 2 + nthr - 1) / nthr;  // pair slots per thread
                        if (PP > 1 && (nt + 1) / 2 <= (PP - 1) * nthr)  // uniform: every thread flies this plane
                            adj_panels<(PP > 1 ? PP - 1 : 1)>(pr, sp, sa, nt, P.cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                        else
                            adj_panels<PP>(pr, sp, sa, nt, P.cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                    }
                    const float v[6] = {warp_sum(Lvb.x), warp_sum(Lvb.y), warp_sum(Lvb.z),
                                        warp_sum(Lwp.x), warp_sum(Lwp.y), warp_sum(Lwp.z)};
                    if (lane == 0) put_part(sh.part[par][warp], v);
                    __syncthreads();
                    if (warp == 0) {
                        sum_parts<W>(sh.part[par], &Lvb, &Lwp);
                        pg::step_pre_adj(P, st, pr, Lvb, Lwp, LR, L0, J);
                        if (j == k) L0.pos = L0.pos + Lb_pos;
                        Lnext = L0;
                    }
                    par ^= 1;
                }
                if (sg >= 1) {  // the rest of segment sg - 1
                    if (warp == 1) rebuild(sg - 1, len, a.K, enext);
                    __syncthreads();
                    if (warp == 2) pre(sg - 1, len > 0 ? len - 1 : 0, a.K, enext);
                    __syncthreads();
                }
            }
        } else
        for (int sg = k / a.K; sg >= 0; sg--) {
            const int j0 = sg * a.K, j1 = min(j0 + a.K - 1, k);
            // recompute the segment
            FSt cur, after;
            pg::Pre<float> pr;
            if (scalar) {
                cur = load_state16(ck + sg * kCkFloats);
                pg::step_pre(P, cur, pr);
                if (SOLO && tid == 0) publish(sh.pre, pr, 0.f);
            }
            __syncthreads();  // staging / the previous segment's last use of the buffers is complete
            int to_chunk = kChunk - j0 % kChunk;
            if (a.fsum) {
                // the forward pass kept every step's force and torque: the states follow from the
                // checkpoint through the integrator alone (the same arithmetic, so the same states),
                // rebuilt once, by warp 0, for the whole block
                if (warp == 0) {
                    const float* fs = a.fsum + ((size_t)f * a.max_steps + j0) * 8;
                    for (int j = j0; j <= j1; j++) {
                        F3 Fb, Tb;
                        load_fsum(fs + (j - j0) * 8, &Fb, &Tb);
                        if (tid == 0) store_seg(seg + (j - j0) * kSegFloats, cur, Fb, Tb);
                        const FSt nx = pg::step_post(P, cur, pr, Fb, Tb);
                        if (j < j1) {
                            cur = nx;
                            if (--to_chunk == 0) { cur.t = (float)(j + 1) * pg::kDt; to_chunk = kChunk; }
                            pg::rot_rows(cur.q, pr.R);  // step_post reads only the attitude matrix
                        } else {
                            after = nx;
                            if (lane == 0 && j1 == k) store_state16(sh.after, after);
                        }
                    }
                }
            }
            for (int j = j0; j <= j1 && !a.fsum; j++) {
                if (SOLO) subscribe(sh.pre, pr);
                float part[6];
                panel_partial_nt<W>(pr, sp, nt, P.cf, tid, part);
                if (lane == 0) put_part(sh.part[par][warp], part);
                __syncthreads();
                if (scalar) {
                    F3 Fb, Tb;
                    sum_parts<W>(sh.part[par], &Fb, &Tb);
                    if (tid == 0) store_seg(seg + (j - j0) * kSegFloats, cur, Fb, Tb);
                    const FSt nx = pg::step_post(P, cur, pr, Fb, Tb);
                    if (j < j1) {
                        cur = nx;
                        if (--to_chunk == 0) { cur.t = (float)(j + 1) * pg::kDt; to_chunk = kChunk; }
                        pg::step_pre(P, cur, pr);
                        if (SOLO && tid == 0) publish(sh.pre, pr, 0.f);
                    } else {
                        after = nx;
                    }
                }
                par ^= 1;
                if (SOLO) __syncthreads();
            }
            __syncthreads();  // the segment's last entry is visible to every warp
            if (a.fsum && scalar && warp != 0 && j1 == k) after = load_state16(sh.after);
            if (scalar && j1 == k) {
                F3 Fd, Td;
                const FSt before = load_seg(seg + (k - j0) * kSegFloats, &Fd, &Td);
                FSt Lb = zero_state();
                pg::terminate_adj(before, after, kind, Lb, Lnext);
                Lb_pos = Lb.pos;
            }
            // adjoint over the segment
            for (int j = j1; j >= j0; j--) {
                FSt s, L0;
                pg::M3<float> LR;
                float Jw[3][3];
                F3 LFb, LTb;
                if (scalar) {
                    F3 Fb, Tb;
                    s = load_seg(seg + (j - j0) * kSegFloats, &Fb, &Tb);
                    pg::step_pre(P, s, pr, Jw);
                    L0 = zero_state();
#pragma unroll
                    for (int r = 0; r < 3; r++)
#pragma unroll
                        for (int q = 0; q < 3; q++) LR.a[r][q] = 0.f;
                    pg::step_post_adj(P, s, pr, Fb, Tb, Lnext, L0, &LFb, &LTb, LR, LP);
                    if (SOLO && tid == 0) {
                        publish(sh.pre, pr, 0.f);
                        sh.adj[0] = LFb.x; sh.adj[1] = LFb.y; sh.adj[2] = LFb.z;
                        sh.adj[3] = LTb.x; sh.adj[4] = LTb.y; sh.adj[5] = LTb.z;
                    }
                }
                if (SOLO) {
                    __syncthreads();
                    subscribe(sh.pre, pr);
                    LFb = pg::v3(sh.adj[0], sh.adj[1], sh.adj[2]);
                    LTb = pg::v3(sh.adj[3], sh.adj[4], sh.adj[5]);
                }
                F3 Lvb, Lwp;
                {
                    constexpr int PP = (kNtMax / 2 + nthr - 1) / nthr;  // pair slots per thread
                    if (PP > 1 && (nt + 1) / 2 <= (PP - 1) * nthr)  // uniform: every thread flies this plane
                        adj_panels<(PP > 1 ? PP - 1 : 1)>(pr, sp, sa, nt, P.cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                    else
                        adj_panels<PP>(pr, sp, sa, nt, P.cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                }
                const float v[6] = {warp_sum(Lvb.x), warp_sum(Lvb.y), warp_sum(Lvb.z),
                                    warp_sum(Lwp.x), warp_sum(Lwp.y), warp_sum(Lwp.z)};
                if (lane == 0) put_part(sh.part[par][warp], v);
                __syncthreads();
                if (scalar) {
                    sum_parts<W>(sh.part[par], &Lvb, &Lwp);
                    pg::step_pre_adj(P, s, pr, Lvb, Lwp, LR, L0, Jw);
                    if (j == k) L0.pos = L0.pos + Lb_pos;
                    Lnext = L0;
                }
                par ^= 1;
            }
            __syncthreads();  // the segment buffer is free for the next recompute
        }
        // release, print variation and staging: re-derived, then their adjoints
        FlightCtx c;
        flight_setup(a, f, c);
        if (scalar) {
            F3 L1rel, wb1;
            (void)pg::release(c.sc, P, c.cg, &L1rel, &wb1);
            pg::release_adj(P, L1rel, wb1, Lnext, LP);
            float Lmass, LI[6];
            pg::printed_adj(P, c.sigma, c.beta, LP, &Lmass, LI);
            if (tid == 0) {
                out[0] = Lmass;
#pragma unroll
                for (int q = 0; q < 6; q++) out[1 + q] = LI[q];
                out[7] = 0.f;
            }
        }
        for (int i = tid; i < nt; i += nthr) {
            const float4 c4 = a.pc[c.off + i], n4 = a.pn[c.off + i];
            F3 Lc, Ln;
            float LA;
            pg::stage_adj(pg::v3(c4.x, c4.y, c4.z), pg::v3(n4.x, n4.y, n4.z), c.cg, c.sc[pg::SC_RHO],
                          c.sc[pg::SC_WP], c.sc[pg::SC_WR], pg::v3(sa[i], sa[kNtMax + i], sa[2 * kNtMax + i]),
                          pg::v3(sa[3 * kNtMax + i], sa[4 * kNtMax + i], sa[5 * kNtMax + i]), sa[6 * kNtMax + i],
                          &Lc, &LA, &Ln);
            float* o = out + 8;
            o[0 * kNtMax + i] = Lc.x; o[1 * kNtMax + i] = Lc.y; o[2 * kNtMax + i] = Lc.z;
            o[3 * kNtMax + i] = LA;
            o[4 * kNtMax + i] = Ln.x; o[5 * kNtMax + i] = Ln.y; o[6 * kNtMax + i] = Ln.z;
        }
    }
    // the longest flights' kernel (LONG) completes before this one does, so what follows on the stream
    // sees both (a no-op when this kernel was not launched as a dependent)
    if (!LONG) asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Exchange area of the grouped reverse pass: per flight of the block, warp 0's published step
// values and each warp's partial sums, and the flights' constants.
template <int W, int M>
struct GroupShared {
    alignas(16) float rcur[M][16];   // pipelined: warp 1's rebuilt state of each flight between steps
    alignas(16) float after[M][16];  // pipelined: the state after each flight's last step (float4 I/O)
    float part[2][W][M][8];          // [parity][warp][flight] 6 partial sums
    float pre[M][8];                 // vb xyz, w xyz
    float adj[M][8];                 // LFb xyz, LTb xyz
    float cf[M];
    int nt[M], k[M], f[M];  // panels, last step (-1: nothing to differentiate), flight (-1: none)
    int next, cnt;          // the block's first flight (order index) and how many it takes
    int rchunk[M];          // pipelined: steps to the next 600-step clock restart
};

// An entry of the pipelined grouped pass (kPEnt floats): the state before a step, the step's body
// force and torque (written by the rebuild) and its step_pre values (written one iteration later):
//   [0..13] pos q vel w t  [16..18] Fb  [19..21] Tb  [24..26] va  [28..30] vb
//   the gust Jacobian J (row-major) in the gaps [14] [15] [22] [23] [27] [31] [32] [33] [34]
constexpr int kPEnt = 36;
constexpr int kPipeGroupMaxK = 60;  // one segment of entries per flight: 4 blocks of 3 warps per SM
__device__ __forceinline__ void put_pent_post(float* e, const FSt& s, F3 F, F3 T) {
    store_state16(e, s);
    store_fsum(e + 16, F, T);
}
__device__ __forceinline__ void put_pent_pre(float* e, const pg::Pre<float>& q, const float (*J)[3]) {
    e[14] = J[0][0]; e[15] = J[0][1]; e[22] = J[0][2];
    e[23] = J[1][0]; e[27] = J[1][1]; e[31] = J[1][2];
    e[32] = J[2][0]; e[33] = J[2][1]; e[34] = J[2][2];
    put3(e + 24, q.va);
    put3(e + 28, q.vb);
}
__device__ __forceinline__ void get_pent(const float* e, FSt& s, F3* F, F3* T, pg::Pre<float>& q, float (*J)[3]) {
    const float4* e4 = reinterpret_cast<const float4*>(e);
    const float4 a = e4[0], b = e4[1], c = e4[2], d = e4[3], f0 = e4[4], f1 = e4[5], v0 = e4[6], v1 = e4[7],
                 j2 = e4[8];
    s.pos = pg::v3(a.x, a.y, a.z);
    s.q[0] = a.w; s.q[1] = b.x; s.q[2] = b.y; s.q[3] = b.z;
    s.vel = pg::v3(b.w, c.x, c.y);
    s.w = pg::v3(c.z, c.w, d.x);
    s.t = d.y;
    J[0][0] = d.z; J[0][1] = d.w;
    *F = pg::v3(f0.x, f0.y, f0.z);
    *T = pg::v3(f0.w, f1.x, f1.y);
    J[0][2] = f1.z; J[1][0] = f1.w;
    q.va = pg::v3(v0.x, v0.y, v0.z);
    J[1][1] = v0.w;
    q.vb = pg::v3(v1.x, v1.y, v1.z);
    J[1][2] = v1.w;
    J[2][0] = j2.x; J[2][1] = j2.y; J[2][2] = j2.z;
}
template <int W, int M>
__host__ __device__ constexpr int group_head_floats() { return (int)((sizeof(GroupShared<W, M>) + 15) / 16 * 4); }

// The reverse pass for up to M flights per block of W warps, when the forward pass kept every
// step's force and torque.  Flights come in k_grad_order's order (longest first): the first
// n_single of them a block each, as their chains set the pass's length, the others M at a time, so
// a block's flights have similar lengths.  The integrator's part of a step -- rebuilding the
// segment, step_pre and its gust Jacobian, the integrator's adjoint and step_pre's -- is scalar
// work along each flight's chain; warp 0 runs it for all M flights at once, lane group g (8 lanes)
// on flight g, so one instruction stream carries M chains.  The panel adjoint of each flight still
// runs on all W warps.
// The flights are aligned by absolute step (their checkpoints are at the same multiples of K): a
// flight joins at its last step and takes no work at the steps after it.  A flight's arithmetic and
// summation order do not depend on the flights beside it, so which flights share a block changes no
// bit of the result.
// PIPE (K <= kPipeGroupMaxK): as in k_grad_reverse's pipelined pass, while warp 0 differentiates
// segment sg, warp 1 rebuilds segment sg - 1 from its checkpoint and the stored forces (one step per
// step, lane group g on flight g, into the slots warp 0 has already read) and warp 2 evaluates each
// rebuilt step's step_pre and gust Jacobian one step behind, so warp 0's chain holds only the
// adjoints of the integrator and of step_pre.
template <int W, int M, bool PIPE>
__global__ void __launch_bounds__(32 * W, (W >= 8 ? 1 : 12 / W)) k_grad_reverse_group(GradArgs a) {
    static_assert(!PIPE || W >= 3, "the pipelined pass needs warps 1 and 2");
    using GS = GroupShared<W, M>;
    static_assert(offsetof(GS, rcur) % 16 == 0 && offsetof(GS, after) % 16 == 0, "states are moved as float4");
    static_assert(M >= 1 && M <= 4, "lane groups of 8 lanes");
    extern __shared__ __align__(16) float smem[];
    GroupShared<W, M>& sh = *reinterpret_cast<GroupShared<W, M>*>(smem);
    float* base = smem + group_head_floats<W, M>();  // per flight: staged panels, then their adjoints
    constexpr int nthr = 32 * W;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 3;            // warp 0: lane group g integrates flight g of the block
    const bool lead = (lane & 7) == 0;  // the group's lane that writes shared memory
    float* segg = base + (size_t)M * 2 * kPanelFloats + (size_t)(g < M ? g : 0) * a.K * kSegFloats;
    for (;;) {
        if (tid == 0) {  // the first n_single tickets take one flight each, the others M
            const int t = atomicAdd(&a.work[1], 1);
            sh.next = a.n_long + (t < a.n_single ? t : a.n_single + (t - a.n_single) * M);
            sh.cnt = t < a.n_single ? 1 : M;
        }
        __syncthreads();
        const int idx0 = sh.next;
        if (idx0 >= a.n_flights) break;
        if (tid < M) {
            const int idx = tid < sh.cnt ? idx0 + tid : a.n_flights;
            int f = -1, kk = -1;
            if (idx < a.n_flights) {
                f = a.order[idx];
                const int kind = a.kind[f];
                if (kind != 0 && kind != 3) kk = a.steps[f] - 1;  // oversize or NaN: constant distance
            }
            sh.f[tid] = f;
            sh.k[tid] = kk;
        }
        __syncthreads();
        int kmax = -1;
#pragma unroll
        for (int m = 0; m < M; m++) kmax = max(kmax, sh.k[m]);
#pragma unroll 1
        for (int m = 0; m < M; m++) {
            const int f = sh.f[m];
            if (f < 0) continue;
            float* out = a.adj + (size_t)f * kAdjStride;
            if (sh.k[m] < 0) {
                for (int i = tid; i < kAdjStride; i += nthr) out[i] = 0.f;
                continue;
            }
            FlightCtx c;
            flight_setup(a, f, c);
            float* sp = base + (size_t)m * 2 * kPanelFloats;
            stage_panels(a, c, sp, tid, nthr);
            for (int i = tid; i < kPanelFloats; i += nthr) sp[kPanelFloats + i] = 0.f;
            if (tid == 0) {
                sh.nt[m] = c.nt;
                sh.cf[m] = a.setup[(size_t)f * kGradSetupFloats + 17];
            }
        }
        // lane group g of warp 0 (and, pipelined, of warps 1 and 2): flight g's constants; warp 0 holds
        // its adjoint state
        const bool grp = g < M && sh.k[g < M ? g : 0] >= 0;
        const bool mine = warp == 0 && grp;
        const bool role = (PIPE ? warp < 3 : warp == 0) && grp;
        const int fg = role ? sh.f[g] : 0, kg = role ? sh.k[g] : -1;
        const int kind = mine ? a.kind[fg] : 0;
        pg::FlightP<float> P;
        if (role) P = setup_flightp(a, fg);
        const float* ck = a.ck + (size_t)fg * a.nck * kCkFloats;
        const float* fsf = a.fsum + (size_t)fg * a.max_steps * 8;
        pg::LamP<float> LP;
        LP.mass = LP.invmass = 0.f;
#pragma unroll
        for (int q = 0; q < 6; q++) LP.I[q] = 0.f;
#pragma unroll
        for (int q = 0; q < 9; q++) LP.invI[q] = 0.f;
        FSt Lnext = zero_state();
        F3 Lb_pos = pg::v3(0.f, 0.f, 0.f);
        int par = 0;
        // every warp: the panel adjoint of step j of each flight still in the air at j, into the
        // step's partial sums
        auto panel_phase = [&](int j) {
#pragma unroll 1
            for (int m = 0; m < M; m++) {
                if (j > sh.k[m]) continue;  // uniform: flight m has ended by step j
                pg::Pre<float> pm;
                subscribe(sh.pre[m], pm);
                const F3 LFb = pg::v3(sh.adj[m][0], sh.adj[m][1], sh.adj[m][2]);
                const F3 LTb = pg::v3(sh.adj[m][3], sh.adj[m][4], sh.adj[m][5]);
                const int nt = sh.nt[m];
                const float cf = sh.cf[m];
                float* sp = base + (size_t)m * 2 * kPanelFloats;
                F3 Lvb, Lwp;
                constexpr int PP = (kNtMax / 2 + nthr - 1) / nthr;  // pair slots per thread
                if (PP > 1 && (nt + 1) / 2 <= (PP - 1) * nthr)  // uniform: every thread flies this plane
                    adj_panels<(PP > 1 ? PP - 1 : 1)>(pm, sp, sp + kPanelFloats, nt, cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                else
                    adj_panels<PP>(pm, sp, sp + kPanelFloats, nt, cf, LFb, LTb, tid, nthr, &Lvb, &Lwp);
                const float v[6] = {warp_sum(Lvb.x), warp_sum(Lvb.y), warp_sum(Lvb.z),
                                    warp_sum(Lwp.x), warp_sum(Lwp.y), warp_sum(Lwp.z)};
                if (lane == 0) put_part(sh.part[par][warp][m], v);
            }
        };
        // warp 0, lane group g: publish the step's (vb, w) and (LFb, LTb) for the panel phase
        auto publish_step = [&](const pg::Pre<float>& pr, F3 LFb, F3 LTb) {
            if (lead) {
                publish(sh.pre[g], pr, 0.f);
                sh.adj[g][0] = LFb.x; sh.adj[g][1] = LFb.y; sh.adj[g][2] = LFb.z;
                sh.adj[g][3] = LTb.x; sh.adj[g][4] = LTb.y; sh.adj[g][5] = LTb.z;
            }
        };
        // warp 0, lane group g: the panels' (Lvb, Lw) summed in warp order, then step_pre's adjoint
        auto finish_step = [&](int j, const FSt& st, const pg::Pre<float>& pr, pg::M3<float>& LR, FSt& L0,
                               const float (*Jw)[3]) {
            float v[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {  // warp order, as sum_parts
                float t = sh.part[par][0][g][q];
#pragma unroll
                for (int w = 1; w < W; w++) t += sh.part[par][w][g][q];
                v[q] = t;
            }
            const F3 Lvb = pg::v3(v[0], v[1], v[2]), Lwp = pg::v3(v[3], v[4], v[5]);
            pg::step_pre_adj(P, st, pr, Lvb, Lwp, LR, L0, Jw);
            if (j == kg) L0.pos = L0.pos + Lb_pos;
            Lnext = L0;
        };
        if constexpr (PIPE) {
            // One segment of entries per flight, reused in place: warp 1 writes each rebuilt entry of
            // segment sg - 1 into a slot whose entry of segment sg warp 0 has already differentiated,
            // so a flight's slots run in reverse from one segment to the next.  slot(s, n) is where
            // entry n of segment s lives: the flight's last segment (Lg steps, rebuilt before its
            // adjoint starts) in slots 0 .. Lg - 1; the one before it in the freed slots, last first,
            // then in Lg .. K - 1; and so on, alternating.
            float* eb = base + (size_t)M * 2 * kPanelFloats;  // [M][K] entries
            const int sLg = kg >= 0 ? kg / a.K : -1;           // flight g's last segment
            const int Lg = kg - sLg * a.K + 1;                 // and its steps
            auto slot = [&](int sgi, int n) {
                const int d = sLg - sgi;
                if (d == 0) return n;
                const int m = (d & 1) ? n : a.K - 1 - n;
                return m < Lg ? Lg - 1 - m : m;
            };
            auto ent = [&](int sgi, int n) {
                return eb + ((size_t)(g < M ? g : 0) * a.K + slot(sgi, n)) * kPEnt;
            };
            auto seg_len = [&](int sgi) {  // steps of flight g in segment sgi
                const int j0 = sgi * a.K;
                return kg >= j0 ? min(a.K, kg - j0 + 1) : 0;
            };
            // the entry of segment sg - 1 that warp 1 rebuilds in iteration i of segment sg's adjoint
            // (j1: the segment's last step of the block): entry i where flight g has no step in sg,
            // else entry i - i0 - 1, one iteration after warp 0 read the entry whose slot it takes (i0:
            // the iteration of the flight's first step in sg)
            auto rb_entry = [&](int sg, int j1, int i) {
                return kg < sg * a.K ? i : i - (j1 - min(j1, kg)) - 1;
            };
            // entries of segment sg - 1 rebuilt in iterations 0 .. i - 1
            auto rb_count = [&](int sg, int j1, int i) {
                return i <= 0 ? 0 : max(0, min(seg_len(sg - 1), rb_entry(sg, j1, i - 1) + 1));
            };
            // warp 1: start rebuilding segment sgi of flight g from its checkpoint
            auto rb_start = [&](int sgi) {
                if (role && lead && seg_len(sgi) > 0) {
                    store_state16(sh.rcur[g], load_state16(ck + (size_t)sgi * kCkFloats));
                    sh.rchunk[g] = kChunk - (sgi * a.K) % kChunk;
                }
            };
            // warp 1: steps n0 .. n1 - 1 of segment sgi, from the state in sh.rcur (the state after
            // the flight's last step into sh.after)
            auto rb_steps = [&](int sgi, int n0, int n1) {
                const int n1g = min(n1, seg_len(sgi));
                if (!role || n0 >= n1g) return;
                FSt cur = load_state16(sh.rcur[g]);
                int to_chunk = sh.rchunk[g];
                pg::Pre<float> pr;
                for (int n = n0; n < n1g; n++) {
                    const int j = sgi * a.K + n;
                    F3 Fb, Tb;
                    load_fsum(fsf + (size_t)j * 8, &Fb, &Tb);
                    if (lead) put_pent_post(ent(sgi, n), cur, Fb, Tb);
                    pg::rot_rows(cur.q, pr.R);  // step_post reads only the attitude matrix
                    const FSt nx = pg::step_post(P, cur, pr, Fb, Tb);
                    if (j == kg) {
                        if (lead) store_state16(sh.after[g], nx);
                    } else {
                        cur = nx;
                        if (--to_chunk == 0) { cur.t = (float)(j + 1) * pg::kDt; to_chunk = kChunk; }  // src/sim.cu:113
                    }
                }
                if (lead) {
                    store_state16(sh.rcur[g], cur);
                    sh.rchunk[g] = to_chunk;
                }
            };
            // warp 2: step_pre and the gust Jacobian of the rebuilt steps n0 .. n1 - 1 of segment sgi
            auto pre_steps = [&](int sgi, int n0, int n1) {
                if (!role) return;
                const int n1g = min(n1, seg_len(sgi));
                for (int n = n0; n < n1g; n++) {
                    float* e = ent(sgi, n);
                    FSt st;
                    F3 Fb, Tb;
                    pg::Pre<float> q;
                    float J[3][3];
                    get_pent(e, st, &Fb, &Tb, q, J);
                    pg::step_pre(P, st, q, J);
                    if (lead) put_pent_pre(e, q, J);
                }
            };
            if (kmax >= 0) {
                const int S = kmax / a.K;
                // prologue: the last segment rebuilt and its step_pre's evaluated
                if (warp == 1) {
                    rb_start(S);
                    __syncwarp();
                    rb_steps(S, 0, a.K);
                }
                __syncthreads();
                if (warp == 2) pre_steps(S, 0, a.K);
                __syncthreads();
                for (int sg = S; sg >= 0; sg--) {
                    const int j0 = sg * a.K, j1 = min(j0 + a.K - 1, kmax), len = j1 - j0 + 1;
                    if (mine && j0 <= kg && kg <= j1) {  // the flight's last step is in this segment
                        FSt before;
                        F3 Fd, Td;
                        pg::Pre<float> qd;
                        float Jd[3][3];
                        get_pent(ent(sg, kg - j0), before, &Fd, &Td, qd, Jd);
                        const FSt after = load_state16(sh.after[g]);
                        FSt Lb = zero_state();
                        pg::terminate_adj(before, after, kind, Lb, Lnext);
                        Lb_pos = Lb.pos;
                    }
                    if (warp == 1 && sg >= 1) {
                        rb_start(sg - 1);
                        __syncwarp();
                    }
                    for (int n = 0; n < len; n++) {
                        const int j = j1 - n;
                        const bool act = mine && j <= kg;
                        FSt st, L0;
                        pg::Pre<float> pr;
                        pg::M3<float> LR;
                        float Jw[3][3];
                        if (act) {
                            F3 Fb, Tb, LFb, LTb;
                            get_pent(ent(sg, j - j0), st, &Fb, &Tb, pr, Jw);
                            pg::rot_rows(st.q, pr.R);
                            pr.w = st.w;
                            L0 = zero_state();
#pragma unroll
                            for (int r = 0; r < 3; r++)
#pragma unroll
                                for (int q = 0; q < 3; q++) LR.a[r][q] = 0.f;
                            pg::step_post_adj(P, st, pr, Fb, Tb, Lnext, L0, &LFb, &LTb, LR, LP);
                            publish_step(pr, LFb, LTb);
                        } else if (warp == 1 && sg >= 1) {
                            const int nb = rb_entry(sg, j1, n);
                            if (nb >= 0) rb_steps(sg - 1, nb, nb + 1);
                        } else if (warp == 2 && sg >= 1 && n >= 1) {  // the entry rebuilt one iteration ago
                            const int nb = rb_entry(sg, j1, n - 1);
                            if (nb >= 0) pre_steps(sg - 1, nb, nb + 1);
                        }
                        __syncthreads();
                        panel_phase(j);
                        __syncthreads();
                        if (act) finish_step(j, st, pr, LR, L0, Jw);
                        par ^= 1;
                    }
                    if (sg >= 1) {  // the rest of segment sg - 1
                        if (warp == 1) rb_steps(sg - 1, rb_count(sg, j1, len), a.K);
                        __syncthreads();
                        if (warp == 2) pre_steps(sg - 1, rb_count(sg, j1, len - 1), a.K);
                    }
                    __syncthreads();  // segment sg - 1 complete before its adjoint
                }
            }
        } else
        for (int sg = kmax < 0 ? -1 : kmax / a.K; sg >= 0; sg--) {
            const int j0 = sg * a.K, j1 = min(j0 + a.K - 1, kmax);
            // each group rebuilds its flight's states over the segment from the checkpoint and the
            // stored forces (the integrator alone)
            FSt after;
            if (mine && j0 <= kg) {
                const int j1g = min(j1, kg);
                FSt cur = load_state16(ck + (size_t)sg * kCkFloats);
                pg::Pre<float> pr;
                pg::rot_rows(cur.q, pr.R);  // step_post reads only the attitude matrix
                int to_chunk = kChunk - j0 % kChunk;
                for (int j = j0; j <= j1g; j++) {
                    F3 Fb, Tb;
                    load_fsum(fsf + (size_t)j * 8, &Fb, &Tb);
                    if (lead) store_seg(segg + (j - j0) * kSegFloats, cur, Fb, Tb);
                    const FSt nx = pg::step_post(P, cur, pr, Fb, Tb);
                    if (j < j1g) {
                        cur = nx;
                        if (--to_chunk == 0) { cur.t = (float)(j + 1) * pg::kDt; to_chunk = kChunk; }  // src/sim.cu:113
                        pg::rot_rows(cur.q, pr.R);
                    } else {
                        after = nx;
                    }
                }
            }
            __syncthreads();  // staging done / the segment's entries visible to their group
            if (mine && j0 <= kg && kg <= j1) {  // the flight's last step is in this segment
                F3 Fd, Td;
                const FSt before = load_seg(segg + (kg - j0) * kSegFloats, &Fd, &Td);
                FSt Lb = zero_state();
                pg::terminate_adj(before, after, kind, Lb, Lnext);
                Lb_pos = Lb.pos;
            }
            for (int j = j1; j >= j0; j--) {
                const bool act = mine && j <= kg;
                FSt st, L0;
                pg::Pre<float> pr;
                pg::M3<float> LR;
                float Jw[3][3];
                if (act) {
                    F3 Fb, Tb, LFb, LTb;
                    st = load_seg(segg + (j - j0) * kSegFloats, &Fb, &Tb);
                    pg::step_pre(P, st, pr, Jw);
                    L0 = zero_state();
#pragma unroll
                    for (int r = 0; r < 3; r++)
#pragma unroll
                        for (int q = 0; q < 3; q++) LR.a[r][q] = 0.f;
                    pg::step_post_adj(P, st, pr, Fb, Tb, Lnext, L0, &LFb, &LTb, LR, LP);
                    publish_step(pr, LFb, LTb);
                }
                __syncthreads();
                panel_phase(j);
                __syncthreads();
                if (act) finish_step(j, st, pr, LR, L0, Jw);
                par ^= 1;
            }
            __syncthreads();  // the segment buffers are free for the next rebuild
        }
        // release, print variation and staging: re-derived, then their adjoints
        if (mine) {
            FlightCtx c;
            flight_setup(a, fg, c);
            F3 L1rel, wb1;
            (void)pg::release(c.sc, P, c.cg, &L1rel, &wb1);
            pg::release_adj(P, L1rel, wb1, Lnext, LP);
            float Lmass, LI[6];
            pg::printed_adj(P, c.sigma, c.beta, LP, &Lmass, LI);
            if (lead) {
                float* out = a.adj + (size_t)fg * kAdjStride;
                out[0] = Lmass;
#pragma unroll
                for (int q = 0; q < 6; q++) out[1 + q] = LI[q];
                out[7] = 0.f;
            }
        }
#pragma unroll 1
        for (int m = 0; m < M; m++) {
            if (sh.k[m] < 0) continue;
            FlightCtx c;
            flight_setup(a, sh.f[m], c);
            const float* sa = base + (size_t)m * 2 * kPanelFloats + kPanelFloats;
            float* o = a.adj + (size_t)sh.f[m] * kAdjStride + 8;
            for (int i = tid; i < c.nt; i += nthr) {
                const float4 c4 = a.pc[c.off + i], n4 = a.pn[c.off + i];
                F3 Lc, Ln;
                float LA;
                pg::stage_adj(pg::v3(c4.x, c4.y, c4.z), pg::v3(n4.x, n4.y, n4.z), c.cg, c.sc[pg::SC_RHO],
                              c.sc[pg::SC_WP], c.sc[pg::SC_WR], pg::v3(sa[i], sa[kNtMax + i], sa[2 * kNtMax + i]),
                              pg::v3(sa[3 * kNtMax + i], sa[4 * kNtMax + i], sa[5 * kNtMax + i]), sa[6 * kNtMax + i],
                              &Lc, &LA, &Ln);
                o[0 * kNtMax + i] = Lc.x; o[1 * kNtMax + i] = Lc.y; o[2 * kNtMax + i] = Lc.z;
                o[3 * kNtMax + i] = LA;
                o[4 * kNtMax + i] = Ln.x; o[5 * kNtMax + i] = Ln.y; o[6 * kNtMax + i] = Ln.z;
            }
        }
        __syncthreads();  // the block's shared state is free for its next flights
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------------------------ per plane: weights and genome contraction
// Tail weights of a plane's distances and the weighted sum of its flights' adjoints (ybar).
constexpr int kWeightThreads = 128;
__global__ void __launch_bounds__(kWeightThreads) k_grad_weights(GradArgs a) {
    __shared__ float w[kGradMaxSeeds], d[kGradMaxSeeds];
    __shared__ float J;
    const int p = blockIdx.x, tid = threadIdx.x, S = a.nseeds;
    const int nt = a.plane_nt[p];
    float* yb = a.ybar + (size_t)p * kAdjStride;
    if (nt <= 0) {  // oversize: the objective is the constant -100
        if (tid == 0 && a.obj) a.obj[p] = -100.f;
        return;
    }
    for (int s = tid; s < S; s += kWeightThreads) d[s] = a.dist[(size_t)p * S + s];
    __syncthreads();
    if (tid == 0) J = pg::objective_weights(d, S, w);
    __syncthreads();
    if (tid == 0 && a.obj) a.obj[p] = J;
    const float* base = a.adj + (size_t)p * S * kAdjStride;
    for (int i = tid; i < 8 + 7 * nt; i += kWeightThreads) {
        // entries 0..7 (mass, I, pad), then 7 panel fields of nt each at stride kNtMax
        const int q = i < 8 ? i : 8 + ((i - 8) / nt) * kNtMax + (i - 8) % nt;
        float acc = 0.f;
        for (int s = 0; s < S; s++) acc += w[s] * base[(size_t)s * kAdjStride + q];
        yb[q] = acc;
    }
}

// Sum of n floats over a block of kGenomeThreads (every thread gets the totals).
constexpr int kGenomeThreads = 128;
template <int N>
__device__ __forceinline__ void block_sum(float v[N], float (*scratch)[N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) scratch[warp][k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) {
        float t = scratch[0][k];
#pragma unroll
        for (int w = 1; w < kGenomeThreads / 32; w++) t += scratch[w][k];
        v[k] = t;
    }
    __syncthreads();
}

// d(objective)/d(gene j) of plane p for block (p * 35 + j): one dual-number pass with tangent
// e_j through mesh -> mass_props -> panels, parallel over vertices and triangles, dotted with
// the plane's ybar.
__global__ void __launch_bounds__(kGenomeThreads) k_grad_genome(GradArgs a) {
    using D = pg::Dual<float>;
    __shared__ D g[kGenomeN];
    __shared__ pg::V3<D> V[kNvMax];
    __shared__ float red[kGenomeThreads / 32][12];
    const int p = blockIdx.x / kGenomeN, j = blockIdx.x - p * kGenomeN, tid = threadIdx.x;
    const int nt = a.plane_nt[p];
    if (nt <= 0) {
        if (tid == 0) a.grad[(size_t)p * kGenomeN + j] = 0.f;
        return;
    }
    if (tid < kGenomeN) g[tid] = D(a.genomes[(size_t)p * kGenomeN + tid], tid == j ? 1.f : 0.f);
    __syncthreads();
    const pg::Topo tp = pg::topology(g);
    for (int i = tid; i < tp.nv; i += kGenomeThreads) V[i] = pg::mesh_vertex(g, tp, i);
    __syncthreads();
    // pass 1: mass and first moment
    float v8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = tid; i < tp.nt; i += kGenomeThreads) {
        D mi;
        pg::V3<D> mc;
        pg::tri_mass(V, tp, i, &mi, &mc);
        v8[0] += mi.v; v8[1] += mi.d; v8[2] += mc.x.v; v8[3] += mc.x.d;
        v8[4] += mc.y.v; v8[5] += mc.y.d; v8[6] += mc.z.v; v8[7] += mc.z.d;
    }
    block_sum<8>(v8, reinterpret_cast<float(*)[8]>(red));
    D m(v8[0], v8[1]), mn;
    pg::V3<D> c = pg::v3(D(v8[2], v8[3]), D(v8[4], v8[5]), D(v8[6], v8[7])), np;
    pg::mass_com(g, &m, &c, &mn, &np);
    // pass 2: inertia about the COM
    D I[6] = {D(0.f), D(0.f), D(0.f), D(0.f), D(0.f), D(0.f)};
    for (int i = tid; i < tp.nt; i += kGenomeThreads) pg::tri_inertia(V, tp, i, c, I);
    float v12[12];
#pragma unroll
    for (int q = 0; q < 6; q++) { v12[2 * q] = I[q].v; v12[2 * q + 1] = I[q].d; }
    block_sum<12>(v12, red);
#pragma unroll
    for (int q = 0; q < 6; q++) I[q] = D(v12[2 * q], v12[2 * q + 1]);
    pg::inertia_finish(mn, np, c, I);
    // panels dotted with ybar
    const float* yb = a.ybar + (size_t)p * kAdjStride;
    const float* yc = yb + 8;
    float acc[1] = {0.f};
    for (int t = tid; t < nt; t += kGenomeThreads) {
        pg::V3<D> ct, n;
        D A;
        pg::panel(V, tp, c, t, &ct, &A, &n);
        acc[0] += yc[t] * ct.x.d + yc[kNtMax + t] * ct.y.d + yc[2 * kNtMax + t] * ct.z.d + yc[3 * kNtMax + t] * A.d +
                  yc[4 * kNtMax + t] * n.x.d + yc[5 * kNtMax + t] * n.y.d + yc[6 * kNtMax + t] * n.z.d;
    }
    block_sum<1>(acc, reinterpret_cast<float(*)[1]>(red));
    if (tid == 0) {
        float r = acc[0] + yb[0] * m.d;
#pragma unroll
        for (int q = 0; q < 6; q++) r += yb[1 + q] * I[q].d;
        a.grad[(size_t)p * kGenomeN + j] = r;
    }
}

}  // namespace

// Warps per flight of the reverse kernel.
constexpr int kRevW = GRAD_REV_WARPS;
constexpr bool kSolo = GRAD_SOLO != 0;

size_t grad_reverse_smem(int K) {
    return ((size_t)shared_head_floats<kRevW>() + 2 * kPanelFloats + (size_t)K * kSegFloats) * sizeof(float);
}
// The pipelined pass keeps two segments of rebuilt steps.
size_t grad_reverse_long_smem(int K) {
    return ((size_t)shared_head_floats<kRevW>() + 2 * kPanelFloats + (size_t)2 * K * kEntFloats) * sizeof(float);
}
bool grad_long_pass(int K) { return kSolo && kRevW >= 3 && K <= kPipeMaxK; }

// Flights and warps per block of the grouped reverse pass, and whether it runs pipelined at
// interval K.  Three warps at 168 registers and two flights' panels and entries (55 KB at K = 60)
// make 4 blocks, 8 flights, per SM.
constexpr int kRevGroup = GRAD_REV_GROUP;
constexpr int kGroupW = GRAD_GROUP_WARPS;
bool grad_group_pipe(int K) { return kGroupW >= 3 && K <= kPipeGroupMaxK; }
size_t grad_reverse_group_smem(int K) {
    const size_t per_flight = grad_group_pipe(K) ? 2 * kPanelFloats + (size_t)K * kPEnt
                                                 : 2 * kPanelFloats + (size_t)K * kSegFloats;
    return ((size_t)group_head_floats<kGroupW, kRevGroup>() + (size_t)kRevGroup * per_flight) * sizeof(float);
}
int grad_group_size(int K) { return kRevGroup > 1 && K <= kPipeMaxK ? kRevGroup : 1; }
using RevKernel = void (*)(GradArgs);
RevKernel grad_group_kernel(int K) {
    return grad_group_pipe(K) ? k_grad_reverse_group<kGroupW, kRevGroup, true>
                              : k_grad_reverse_group<kGroupW, kRevGroup, false>;
}

cudaError_t grad_configure(int K, int rev_grid[2], int nsm) {
    cudaError_t e = cudaFuncSetAttribute(k_grad_reverse<kRevW, kSolo, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_reverse_smem(K));
    if (e != cudaSuccess) return e;
    if (grad_long_pass(K)) {
        e = cudaFuncSetAttribute(k_grad_reverse<kRevW, kSolo, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)grad_reverse_long_smem(K));
        if (e != cudaSuccess) return e;
    }
    int br = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&br, k_grad_reverse<kRevW, kSolo, false>, 32 * kRevW,
                                                      grad_reverse_smem(K));
    if (e != cudaSuccess) return e;
    rev_grid[0] = (br > 0 ? br : 1) * nsm;
    rev_grid[1] = 0;
    if (grad_group_size(K) > 1) {
        e = cudaFuncSetAttribute(grad_group_kernel(K), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)grad_reverse_group_smem(K));
        if (e != cudaSuccess) return e;
        br = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&br, grad_group_kernel(K), 32 * kGroupW,
                                                          grad_reverse_group_smem(K));
        if (e != cudaSuccess) return e;
        rev_grid[1] = (br > 0 ? br : 1) * nsm;
    }
    return cudaSuccess;
}

cudaError_t launch_grad(const GradArgs& a, const FlightArgs& fwd, int nsm, const int fwd_bps[2], const int rev_grid[2],
                        cudaStream_t s, cudaEvent_t mid) {
    const bool grouped = a.group > 1;
    if (grouped && (a.group != kRevGroup || !a.fsum || rev_grid[1] <= 0)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.work, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_grad_setup<<<(a.n_flights + 127) / 128, 128, 0, s>>>(a);
    e = launch_grad_forward(fwd, nsm, fwd_bps, s);
    if (e != cudaSuccess) return e;
    k_grad_order<<<1, kOrderThreads, 0, s>>>(a.steps, a.n_flights, a.order);
    if (mid) cudaEventRecord(mid, s);
    if (a.n_long > 0) {
        // the longest flights' pipelined pass first; the other flights' kernel is its programmatic
        // dependent, so it starts once those blocks are resident and fills the rest of the GPU
        k_grad_reverse<kRevW, kSolo, true><<<a.n_long, 32 * kRevW, grad_reverse_long_smem(a.K), s>>>(a);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grouped ? rev_grid[1] : rev_grid[0]);
        cfg.blockDim = dim3(32 * (grouped ? kGroupW : kRevW));
        cfg.dynamicSmemBytes = grouped ? grad_reverse_group_smem(a.K) : grad_reverse_smem(a.K);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = grouped ? cudaLaunchKernelEx(&cfg, grad_group_kernel(a.K), a)
                    : cudaLaunchKernelEx(&cfg, k_grad_reverse<kRevW, kSolo, false>, a);
        if (e != cudaSuccess) return e;
    } else if (grouped) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(rev_grid[1]);
        cfg.blockDim = dim3(32 * kGroupW);
        cfg.dynamicSmemBytes = grad_reverse_group_smem(a.K);
        cfg.stream = s;
        e = cudaLaunchKernelEx(&cfg, grad_group_kernel(a.K), a);
        if (e != cudaSuccess) return e;
    } else {
        k_grad_reverse<kRevW, kSolo, false><<<rev_grid[0], 32 * kRevW, grad_reverse_smem(a.K), s>>>(a);
    }
    k_grad_weights<<<a.pop, kWeightThreads, 0, s>>>(a);
    k_grad_genome<<<a.pop * kGenomeN, kGenomeThreads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pe
