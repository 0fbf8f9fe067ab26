// pe_flight.cu -- the 600 Hz 6DOF flight of every (plane, scenario) pair (src/sim.cu:55-212).
//
// Mapping.  A group of LPF lanes (16 or 32) flies one flight at a time; a warp holds 32/LPF
// groups.  Each group pulls flights from a global queue (one atomic per flight), stages the
// flight's panels once into shared memory with the print-warp normal already applied (it is
// constant over a flight: it depends on the panel, the CG shift and the scenario only), and
// then steps: rotate panels to world, relative flow with rotation and gusts, normal force and
// skin friction per panel, group-wide sum of force and torque, and the integrator, which every
// lane of the group evaluates redundantly so no lane waits and no block barrier is needed.
//
// Reduction order.  The reference sums panels with 128 threads, panel t on thread t % 128,
// then a shuffle-down tree inside each warp, then a serial sum of the 4 warp totals
// (src/sim.cu:134-176).  Lane j of a group keeps one accumulator set per virtual thread
// j + LPF*m (m < 128/LPF) and the group reduces those sets along the same tree, so each sum
// rounds exactly as the reference's does.  The transposed shuffle reduction halves the number
// of live values at every level, so all 24 (virtual warp, component) sums cost 31 shuffles.
//
// Chunking.  A launch advances flights by at most `step_end - step_begin` steps; flights still
// airborne are appended to the next launch's list and their state is saved (64 B).  The clock
// restarts at every multiple of 600 steps, as the reference's 600-step launches do
// (src/sim.cu:113), whatever launch length is chosen here.
#include "pe_internal.cuh"

namespace pe {

// Per-flight constants held in registers for the whole flight.
struct FlightConst {
    float mass, invmass;
    float I[6];
    float invI[9];
    float air_rho, skin_cf;
    float phase, gust, base_x, base_y;
    vec3 cg;
    float warp_pitch, warp_roll;
};

__device__ __forceinline__ int flight_env_seed(const FlightArgs& a, int p, int s) {
    return (int)((uint32_t)a.seeds[s] + (a.vary ? (uint32_t)p * 7919u : 0u));
}

__device__ __forceinline__ void flight_setup(const FlightArgs& a, int p, int s, FlightConst* fc,
                                             MassProps* pmp_out, Scenario* sc_out) {
    const int env_seed = flight_env_seed(a, p, s);
    Scenario sc;
    scenario_desc(env_seed, &sc);
    MassProps src;
    const float* m = a.plane_mp + (size_t)p * kMpN;
    src.mass = m[0]; src.invmass = m[1]; src.com = mk3(m[2], m[3], m[4]);
    for (int k = 0; k < 6; k++) src.I[k] = m[5 + k];
    for (int k = 0; k < 9; k++) src.invI[k] = m[11 + k];
    MassProps pmp; vec3 cg;
    printed_mass_props(src, sc, &pmp, &cg);
    fc->mass = pmp.mass; fc->invmass = pmp.invmass;
    for (int k = 0; k < 6; k++) fc->I[k] = pmp.I[k];
    for (int k = 0; k < 9; k++) fc->invI[k] = pmp.invI[k];
    fc->air_rho = sc.v[S_AIR_RHO]; fc->skin_cf = sc.v[S_SKIN_CF];
    fc->phase = seed_phase(env_seed);
    fc->gust = sc.v[S_GUST]; fc->base_x = sc.v[S_BASE_X]; fc->base_y = sc.v[S_BASE_Y];
    fc->cg = cg;
    fc->warp_pitch = sc.v[S_WARP_PITCH]; fc->warp_roll = sc.v[S_WARP_ROLL];
    if (pmp_out) *pmp_out = pmp;
    if (sc_out) *sc_out = sc;
}

// Stage panels with the print-warped unit normal (src/sim.cu:135-143).
template <int LPF>
__device__ __forceinline__ void stage_panels(const FlightArgs& a, int p, int nt, int j, const FlightConst& fc,
                                             float4* s_rb, float4* s_nb) {
    const int off = a.plane_off[p];
    for (int i = j; i < nt; i += LPF) {
        float4 c4 = a.pc[off + i], n4 = a.pn[off + i];
        vec3 rb = vsub(mk3(c4.x, c4.y, c4.z), fc.cg);
        vec3 nb = mk3(n4.x, n4.y, n4.z);
        float ar = fc.warp_roll * fmaxf(-1.f, fminf(1.f, rb.y / 0.125f));
        float ap = fc.warp_pitch * fmaxf(-1.f, fminf(1.f, rb.x / 0.125f));
        vec3 nr = mk3(nb.x, nb.y - ar * nb.z, nb.z + ar * nb.y);
        nb = vnorm(mk3(nr.x + ap * nr.z, nr.y, nr.z - ap * nr.x));
        s_rb[i] = make_float4(rb.x, rb.y, rb.z, c4.w);
        s_nb[i] = make_float4(nb.x, nb.y, nb.z, 0.0f);
    }
}

// Group-wide sum of the per-virtual-thread accumulators in the reference's order.
// acc[m][c]: virtual thread j + LPF*m, component c (F xyz, T xyz).  out[6] on every lane.
template <int LPF>
__device__ __forceinline__ void reduce_exact(float (&acc)[128 / LPF][6], unsigned mask, int j, float out[6]) {
    // 1) tree levels that stay inside one physical lane (LPF = 16: offset 16 pairs virtual
    //    lanes j and j + 16 of the same virtual warp) -> 4 virtual warps x 8 slots (6 used)
    float v[32];
#pragma unroll
    for (int vw = 0; vw < 4; vw++) {
#pragma unroll
        for (int c = 0; c < 8; c++) {
            float x = 0.0f;
            if (c < 6) {
                if (LPF == 32) x = acc[vw][c];
                else x = acc[2 * vw][c] + acc[2 * vw + 1][c];
            }
            v[vw * 8 + c] = x;
        }
    }
    // 2) cross-lane levels, offsets LPF/2 .. 1; each level halves the live values
#pragma unroll
    for (int lv = 0; lv < 5; lv++) {
        const int m = (LPF / 2) >> lv;
        if (m >= 1) {
            const int n = 32 >> lv;
            const bool up = (j & m) != 0;
#pragma unroll
            for (int i = 0; i < n / 2; i++) {
                float send = up ? v[i] : v[i + n / 2];
                float keep = up ? v[i + n / 2] : v[i];
                float recv = __shfl_xor_sync(mask, send, m, LPF);
                v[i] = keep + recv;
            }
        }
    }
    // 3) lane j holds the sums of value indices j*K + k (k < K), index = vwarp * 8 + component.
    //    Serial sum over the 4 virtual warps, starting from zero as thread 0 does.
    constexpr int K = 32 / LPF;
    constexpr int CPL = 8 / K;
    const int jc = j % CPL;
    float tot[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        float s0 = 0.0f;
#pragma unroll
        for (int vw = 0; vw < 4; vw++) s0 = s0 + __shfl_sync(mask, v[k], vw * CPL + jc, LPF);
        tot[k] = s0;
    }
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = __shfl_sync(mask, tot[c % K], c / K, LPF);
}

// Aerodynamic force and torque of one panel, accumulated into acc (src/sim.cu:135-158).
__device__ __forceinline__ void panel_exact(float4 rbA, float4 n4, vec3 r0, vec3 r1, vec3 r2, vec3 ww,
                                            vec3 vel, vec3 wind, float air_rho, float skin_cf, float* acc) {
    vec3 rb = mk3(rbA.x, rbA.y, rbA.z);
    float A = rbA.w;
    vec3 nb = mk3(n4.x, n4.y, n4.z);
    vec3 rw = mk3(vdot(r0, rb), vdot(r1, rb), vdot(r2, rb));
    vec3 nw = mk3(vdot(r0, nb), vdot(r1, nb), vdot(r2, nb));
    vec3 vr = vsub(vadd(vel, vcross(ww, rw)), wind);
    float V2 = vdot(vr, vr);
    if (V2 < 1e-6f) return;
    float Vm = sqrtf(V2);
    vec3 vh = vscl(vr, 1.0f / Vm);
    float s = vdot(vh, nw);
    float qd = 0.5f * air_rho * V2 * A;
    float cn = PE_CN_SLOPE * s * sqrtf(fmaxf(0.f, 1.f - s * s)) + 2.0f * s * fabsf(s);
    vec3 f = vscl(nw, -qd * cn);
    vec3 tang = vsub(vh, vscl(nw, s));
    f = vsub(f, vscl(tang, qd * skin_cf));
    vec3 tq = vcross(rw, f);
    acc[0] = acc[0] + f.x; acc[1] = acc[1] + f.y; acc[2] = acc[2] + f.z;
    acc[3] = acc[3] + tq.x; acc[4] = acc[4] + tq.y; acc[5] = acc[5] + tq.z;
}

// Aerodynamic sums of one step over the staged panels (all lanes of the group get them).
template <int LPF>
__device__ __forceinline__ void aero_sums(const float4* s_rb, const float4* s_nb, int nt, int j, unsigned mask,
                                          vec3 r0, vec3 r1, vec3 r2, vec3 ww, vec3 vel, vec3 wind,
                                          float air_rho, float skin_cf, float out[6]) {
    constexpr int NS = 128 / LPF;
    float acc[NS][6];
#pragma unroll
    for (int m = 0; m < NS; m++)
#pragma unroll
        for (int c = 0; c < 6; c++) acc[m][c] = 0.0f;
    for (int base = 0; base < nt; base += 128) {
#pragma unroll
        for (int m = 0; m < NS; m++) {
            const int i = base + m * LPF + j;
            if (i < nt) panel_exact(s_rb[i], s_nb[i], r0, r1, r2, ww, vel, wind, air_rho, skin_cf, acc[m]);
        }
    }
    reduce_exact<LPF>(acc, mask, j, out);
}

// Integrator and termination, src/sim.cu:177-204.  Returns 1 when the flight ends at `step`.
__device__ __forceinline__ int integrate(const FlightConst& fc, vec3 r0, vec3 r1, vec3 r2, const float sum[6],
                                         FlightState& st, int step, int max_steps, float* fit) {
    // sum[] already holds ((0 + W0) + W1) + W2) + W3, thread 0's serial order
    vec3 Fs = mk3(sum[0], sum[1], sum[2]), Ts = mk3(sum[3], sum[4], sum[5]);
    Fs.z -= fc.mass * PE_GRAV;
    vec3 wb = st.wb, vel = st.vel, pos = st.pos;
    vec3 tb = mk3(r0.x * Ts.x + r1.x * Ts.y + r2.x * Ts.z,
                  r0.y * Ts.x + r1.y * Ts.y + r2.y * Ts.z,
                  r0.z * Ts.x + r1.z * Ts.y + r2.z * Ts.z);
    vec3 Iw = mk3(fc.I[0] * wb.x + fc.I[3] * wb.y + fc.I[4] * wb.z,
                  fc.I[3] * wb.x + fc.I[1] * wb.y + fc.I[5] * wb.z,
                  fc.I[4] * wb.x + fc.I[5] * wb.y + fc.I[2] * wb.z);
    vec3 gyro = vcross(wb, Iw);
    vec3 tq = vsub(tb, gyro);
    vec3 dw = mk3(fc.invI[0] * tq.x + fc.invI[1] * tq.y + fc.invI[2] * tq.z,
                  fc.invI[3] * tq.x + fc.invI[4] * tq.y + fc.invI[5] * tq.z,
                  fc.invI[6] * tq.x + fc.invI[7] * tq.y + fc.invI[8] * tq.z);
    wb = vadd(wb, vscl(dw, PE_DT));
    float wl = vlen(wb);
    if (wl > 150.f) wb = vscl(wb, 150.f / wl);
    vel = vadd(vel, vscl(Fs, fc.invmass * PE_DT));
    float vl = vlen(vel);
    if (vl > 60.f) vel = vscl(vel, 60.f / vl);
    pos = vadd(pos, vscl(vel, PE_DT));
    quat4 q = st.q;
    quat4 dq = qmul(q, mkq(0, wb.x, wb.y, wb.z));
    st.q = qnormalize(mkq(q.w + 0.5f * dq.w * PE_DT, q.x + 0.5f * dq.x * PE_DT,
                          q.y + 0.5f * dq.y * PE_DT, q.z + 0.5f * dq.z * PE_DT));
    st.vel = vel; st.wb = wb; st.pos = pos; st.t += PE_DT;
    int bad = !(pos.x == pos.x && vel.x == vel.x);
    if (pos.z <= 0.0f || bad || fabsf(pos.y) > 300.f || pos.x < -50.f) {
        *fit = bad ? -10.0f : pos.x;
        return 1;
    } else if (step == max_steps - 1) {
        *fit = pos.x;
        return 1;
    }
    return 0;
}

// One full step from st (clock restart included).  sum[6] receives the aerodynamic sums.
template <int LPF>
__device__ __forceinline__ int flight_step(const FlightConst& fc, const float4* s_rb, const float4* s_nb, int nt,
                                           int j, unsigned mask, FlightState& st, int step, int max_steps,
                                           float* fit, float sum[6]) {
    if (step > 0 && step % kChunk == 0) st.t = step * PE_DT;
    vec3 r0, r1, r2;
    qrows(st.q, &r0, &r1, &r2);
    vec3 wb = st.wb;
    vec3 ww = mk3(vdot(r0, wb), vdot(r1, wb), vdot(r2, wb));
    vec3 wind = wind_at(st.pos, st.t, fc.phase, fc.gust, fc.base_x, fc.base_y);
    aero_sums<LPF>(s_rb, s_nb, nt, j, mask, r0, r1, r2, ww, st.vel, wind, fc.air_rho, fc.skin_cf, sum);
    return integrate(fc, r0, r1, r2, sum, st, step, max_steps, fit);
}

template <int LPF>
__device__ __forceinline__ unsigned group_mask(int lane) {
    return LPF == 32 ? 0xffffffffu : (0xffffu << (lane & 16));
}

// Persistent flight kernel: groups pull flights until the list is exhausted.
template <int LPF>
__global__ void __launch_bounds__(256) k_flight(FlightArgs a) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int j = lane % LPF;
    const int slot = threadIdx.x / LPF;
    float4* s_rb = smem + (size_t)slot * 2 * kNtMax;
    float4* s_nb = s_rb + kNtMax;
    const unsigned mask = group_mask<LPF>(lane);
    const int leader = lane - j;
    const int n_work = a.active_in ? *a.n_active_in : a.n_flights;

    while (true) {
        int f = 0;
        if (j == 0) f = atomicAdd(a.work, 1);
        f = __shfl_sync(mask, f, leader);
        if (f >= n_work) break;
        const int flight = a.active_in ? a.active_in[f] : f;
        const int p = flight / a.nseeds, s = flight - p * a.nseeds;
        const int nt = a.plane_nt[p];

        FlightConst fc;
        MassProps pmp;
        Scenario sc;
        flight_setup(a, p, s, &fc, &pmp, &sc);
        FlightState st;
        if (a.step_begin == 0) {
            if (nt <= 0) {  // oversize: hard negative, no steps (src/sim.cu:108-109)
                if (j == 0) { a.dist[flight] = -100.0f; a.steps[flight] = 0; }
                continue;
            }
            release(sc, pmp, fc.cg, &st);
        } else {
            st = a.state[flight];
        }
        __syncwarp(mask);  // the previous flight's panels are no longer read
        stage_panels<LPF>(a, p, nt, j, fc, s_rb, s_nb);
        __syncwarp(mask);

        const int end = min(a.step_end, a.max_steps);
        int step = st.step;
        int done = 0;
        float fit = 0.0f;
        float sum[6];
        for (; step < end; step++) {
            done = flight_step<LPF>(fc, s_rb, s_nb, nt, j, mask, st, step, a.max_steps, &fit, sum);
            if (done) break;
        }
        if (done) {
            if (j == 0) { a.dist[flight] = fit; a.steps[flight] = step + 1; }
        } else if (j == 0 && a.active_out) {
            st.step = step;
            a.state[flight] = st;
            int k = atomicAdd(a.n_active_out, 1);
            a.active_out[k] = flight;
        }
    }
}

// Teacher-forced single step (parity tests): group g steps flight g from state_in[g].
template <int LPF>
__global__ void __launch_bounds__(256) k_debug_step(FlightArgs a, const FlightState* state_in,
                                                    FlightState* state_out, float* FT, int* done_out,
                                                    float* fit_out, int step) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int j = lane % LPF;
    const int slot = threadIdx.x / LPF;
    float4* s_rb = smem + (size_t)slot * 2 * kNtMax;
    float4* s_nb = s_rb + kNtMax;
    const unsigned mask = group_mask<LPF>(lane);
    const int flight = blockIdx.x * (blockDim.x / LPF) + slot;
    if (flight >= a.n_flights) return;
    const int p = flight / a.nseeds, s = flight - p * a.nseeds;
    const int nt = a.plane_nt[p];
    FlightConst fc;
    flight_setup(a, p, s, &fc, nullptr, nullptr);
    stage_panels<LPF>(a, p, nt, j, fc, s_rb, s_nb);
    __syncwarp(mask);
    FlightState st = state_in[flight];
    float fit = 0.0f, sum[6];
    int done = flight_step<LPF>(fc, s_rb, s_nb, nt, j, mask, st, step, a.max_steps, &fit, sum);
    if (j == 0) {
        state_out[flight] = st;
        for (int c = 0; c < 6; c++) FT[flight * 6 + c] = sum[c];
        done_out[flight] = done;
        fit_out[flight] = fit;
    }
}

__global__ void k_debug_release(FlightArgs a, FlightState* out) {
    const int flight = blockIdx.x * blockDim.x + threadIdx.x;
    if (flight >= a.n_flights) return;
    const int p = flight / a.nseeds, s = flight - p * a.nseeds;
    FlightConst fc; MassProps pmp; Scenario sc;
    flight_setup(a, p, s, &fc, &pmp, &sc);
    FlightState st;
    release(sc, pmp, fc.cg, &st);
    out[flight] = st;
}

// ---------------------------------------------------------------- host-side launch helpers
size_t flight_smem_bytes(const FlightShape& sh) {
    return (size_t)(sh.warps * 32 / sh.lanes) * 2 * kNtMax * sizeof(float4);
}

template <int LPF>
static const void* flight_fn() { return (const void*)&k_flight<LPF>; }

int flight_blocks_per_sm(const FlightShape& sh) {
    const void* fn = sh.lanes == 16 ? flight_fn<16>() : flight_fn<32>();
    size_t smem = flight_smem_bytes(sh);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, sh.warps * 32, smem) != cudaSuccess) return 0;
    return nb;
}

cudaError_t launch_flight(const FlightArgs& a, const FlightShape& sh, int grid, cudaStream_t s) {
    size_t smem = flight_smem_bytes(sh);
    const void* fn = sh.lanes == 16 ? flight_fn<16>() : flight_fn<32>();
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (sh.lanes == 16) k_flight<16><<<grid, sh.warps * 32, smem, s>>>(a);
    else if (sh.lanes == 32) k_flight<32><<<grid, sh.warps * 32, smem, s>>>(a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_debug_step(const FlightArgs& a, const FlightState* state_in, FlightState* state_out,
                              float* FT, int* done, float* fit, int step, int lanes, cudaStream_t s) {
    const int threads = 128;
    const int per_block = threads / lanes;
    const int grid = (a.n_flights + per_block - 1) / per_block;
    const size_t smem = (size_t)per_block * 2 * kNtMax * sizeof(float4);
    if (lanes == 16) {
        cudaFuncSetAttribute((const void*)&k_debug_step<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_debug_step<16><<<grid, threads, smem, s>>>(a, state_in, state_out, FT, done, fit, step);
    } else {
        cudaFuncSetAttribute((const void*)&k_debug_step<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_debug_step<32><<<grid, threads, smem, s>>>(a, state_in, state_out, FT, done, fit, step);
    }
    return cudaGetLastError();
}

cudaError_t launch_debug_release(const FlightArgs& a, FlightState* out, cudaStream_t s) {
    k_debug_release<<<(a.n_flights + 127) / 128, 128, 0, s>>>(a, out);
    return cudaGetLastError();
}

}  // namespace pe
