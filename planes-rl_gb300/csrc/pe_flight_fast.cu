// pe_flight_fast.cu -- the flight step in the body frame (the throughput formulation).
//
// Same physics as src/sim.cu:129-204, rearranged for fewer operations per panel:
//   * the air velocity is rotated into the body frame once per step,
//       v_b = R^T (vel - wind),  and per panel  vr = v_b + wb x rb
//     instead of rotating every panel's position and normal into the world frame
//     (R^T (ww x R rb) = wb x rb for a rotation R);
//   * with vh = vr / |vr| and s = vh . nb the panel force
//       f = -qd cn nb - qd cf (vh - s nb) = a nb + b vr,
//       a = -qd (cn - cf s),  b = -qd cf / |vr|,
//     so neither vh nor the tangential vector is formed; 1/|vr| is one rsqrt;
//   * 0.5 rho A is folded into the staged panel once per flight;
//   * force and torque sums stay in the body frame: the integrator needs the body torque and
//     rotates only the total force to the world frame;
//   * two panels share every FP32 instruction (packed f32x2 add/mul/fma of sm_103a), read from
//     a pair-interleaved shared-memory layout so each 128-bit load yields two packed operands;
//     torque is accumulated as the two halves of the cross product and subtracted once per step,
//     so no packed negation is needed.
// About 25 instructions per panel-step against about 80 in the reference's form.  A panel whose
// relative flow is below 1e-3 m/s adds its (vanishing, < 1e-9 of the weight) force instead of
// being skipped.  Results differ from the reference arithmetic in rounding only; the parity
// tests bound the flight-level effect.
//
// Summation order is fixed by panel index, not by the execution shape: panel i belongs to pair
// q = i / 2 (even panels in the low half, odd in the high half), pair q to virtual lane
// v = q % 32; each virtual lane sums its pairs in order, adds its odd to its even partial sum, and
// the 32 virtual lanes reduce along one xor tree, so every shape (16 or 32 lanes per flight, any
// chunk length or grid) is bit-identical.  Every lane of a flight makes the same number of pair
// passes, ceil(ceil(nt / 2) / lanes): 11 for a 344-panel plane at 16 lanes (12 in a layout of
// 64-panel rows).  Passes beyond the plane's pairs read zero panels, whose force and torque are
// exact zeros; the partial sums start at +0 and in round-to-nearest a sum is -0 only when both
// terms are, so adding them changes no bit and the shapes still agree.
#include "pe_f32x2.cuh"
#include "pe_internal.cuh"

namespace pe {

struct FastConst {
    float mass, invmass;
    float I[6];
    float invI[9];
    float skin_cf;
    float phase, gust, base_x, base_y;
};

__device__ __forceinline__ void fast_setup(const FlightArgs& a, int p, int s, FastConst* fc, vec3* cg_out,
                                           float* air_rho, float* warp_pitch, float* warp_roll, MassProps* pmp_out,
                                           Scenario* sc_out) {
    const int env_seed = (int)((uint32_t)a.seeds[s] + (a.vary ? (uint32_t)p * 7919u : 0u));
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
    fc->skin_cf = sc.v[S_SKIN_CF];
    fc->phase = seed_phase(env_seed);
    fc->gust = sc.v[S_GUST]; fc->base_x = sc.v[S_BASE_X]; fc->base_y = sc.v[S_BASE_Y];
    *cg_out = cg;
    *air_rho = sc.v[S_AIR_RHO];
    *warp_pitch = sc.v[S_WARP_PITCH];
    *warp_roll = sc.v[S_WARP_ROLL];
    if (pmp_out) *pmp_out = pmp;
    if (sc_out) *sc_out = sc;
}

// Explicitly rounded arithmetic: the compiler may neither contract nor reorder these, so the
// step is bit-identical in every template instance and execution shape.
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dot_(vec3 a, vec3 b) { return fma_(a.z, b.z, fma_(a.y, b.y, mul_(a.x, b.x))); }
__device__ __forceinline__ float len_(vec3 a) { return __fsqrt_rn(dot_(a, a)); }

// Staged panel: (rb xyz, 0.5 rho A), (print-warped unit normal xyz, 0); src/sim.cu:135-143.
static __device__ __noinline__ void fast_stage_one(float4 c4, float4 n4, vec3 cg, float half_rho, float warp_pitch,
                                                   float warp_roll, float4* oa, float4* ob) {
    const vec3 rb = mk3(sub_(c4.x, cg.x), sub_(c4.y, cg.y), sub_(c4.z, cg.z));
    const float ar = mul_(warp_roll, fmaxf(-1.f, fminf(1.f, mul_(rb.y, 8.0f))));
    const float ap = mul_(warp_pitch, fmaxf(-1.f, fminf(1.f, mul_(rb.x, 8.0f))));
    const vec3 nr = mk3(n4.x, fma_(-ar, n4.z, n4.y), fma_(ar, n4.y, n4.z));
    vec3 nb = mk3(fma_(ap, nr.z, nr.x), nr.y, fma_(-ap, nr.x, nr.z));
    const float l = len_(nb);
    nb = l > 1e-12f ? mk3(__fdiv_rn(nb.x, l), __fdiv_rn(nb.y, l), __fdiv_rn(nb.z, l)) : mk3(0, 0, 1);
    *oa = make_float4(rb.x, rb.y, rb.z, mul_(half_rho, c4.w));
    *ob = make_float4(nb.x, nb.y, nb.z, 0.0f);
}

// Pair-interleaved panel layout of one flight: pair q holds panels 2q (low half) and 2q + 1 (high
// half); virtual lane v owns pairs v, v + 32, v + 64, ...  Slots from panel nt up to the flight's
// last pass are zero panels.
struct PairedPanels {
    float4* a;  // (rbx0, rbx1, rby0, rby1)
    float4* b;  // (rbz0, rbz1, ak0, ak1)   ak = 0.5 rho A
    float4* c;  // (nbx0, nbx1, nby0, nby1)
    float2* d;  // (nbz0, nbz1)
};
// Pair slots of one flight: every pair the passes of LPF lanes read, 176 at 16 lanes, 192 at 32.
template <int LPF>
__host__ __device__ constexpr int slot_pairs() { return LPF * ((kNtMax / 2 + LPF - 1) / LPF); }
template <int LPF>
__host__ __device__ constexpr size_t paired_bytes() {
    return (size_t)slot_pairs<LPF>() * (3 * sizeof(float4) + sizeof(float2));
}
template <int LPF>
__device__ __forceinline__ PairedPanels paired_view(char* base) {
    constexpr int kPairs = slot_pairs<LPF>();
    PairedPanels pp;
    pp.a = (float4*)base;
    pp.b = pp.a + kPairs;
    pp.c = pp.b + kPairs;
    pp.d = (float2*)(pp.c + kPairs);
    return pp;
}

template <int LPF>
__device__ __forceinline__ void fast_stage(const FlightArgs& a, int p, int nt, int j, vec3 cg, float air_rho,
                                           float warp_pitch, float warp_roll, PairedPanels pp) {
    const int off = a.plane_off[p];
    const float half_rho = mul_(0.5f, air_rho);
    const int slots = 2 * LPF * (((nt + 1) / 2 + LPF - 1) / LPF);  // every pair the passes read
    for (int i = j; i < slots; i += LPF) {
        float4 oa = make_float4(0, 0, 0, 0), ob = make_float4(0, 0, 0, 0);
        if (i < nt) fast_stage_one(a.pc[off + i], a.pn[off + i], cg, half_rho, warp_pitch, warp_roll, &oa, &ob);
        const int q = i >> 1, h = i & 1;
        float* pa = (float*)&pp.a[q];
        float* pb = (float*)&pp.b[q];
        float* pc = (float*)&pp.c[q];
        float* pd = (float*)&pp.d[q];
        pa[h] = oa.x; pa[2 + h] = oa.y;
        pb[h] = oa.z; pb[2 + h] = oa.w;
        pc[h] = ob.x; pc[2 + h] = ob.y;
        pd[h] = ob.z;
    }
}

// Gust field (src/common.h:459-467) with explicit rounding.
__device__ __forceinline__ vec3 fast_wind(vec3 p, float t, float s, float gust, float bx, float by) {
    const float a1 = __sinf(add_(fma_(0.9f, p.x, mul_(1.3f, t)), s));
    const float a2 = __sinf(add_(fma_(2.3f, p.z, mul_(2.1f, t)), mul_(1.7f, s)));
    const float a3 = __sinf(add_(fma_(4.1f, p.y, mul_(3.3f, t)), mul_(0.4f, s)));
    const float b1 = __sinf(add_(fma_(1.1f, p.x, mul_(1.7f, t)), mul_(2.2f, s)));
    const float b2 = __sinf(add_(fma_(3.1f, p.z, mul_(2.9f, t)), mul_(0.9f, s)));
    const float c1 = __sinf(add_(fma_(1.4f, p.x, mul_(2.3f, t)), mul_(3.1f, s)));
    const float c2 = __sinf(add_(fma_(2.7f, p.y, mul_(1.9f, t)), mul_(1.2f, s)));
    const float gx = mul_(gust, fma_(0.25f, a3, fma_(0.35f, a2, mul_(0.55f, a1))));
    const float gy = mul_(gust, fma_(0.30f, b2, mul_(0.50f, b1)));
    const float gz = mul_(gust, fma_(0.20f, c2, mul_(0.30f, c1)));
    return mk3(add_(bx, gx), add_(by, gy), gz);
}

// Body->world rotation rows of a unit quaternion (src/common.h:38-43) with explicit rounding.
__device__ __forceinline__ void fast_rows(quat4 q, vec3* r0, vec3* r1, vec3* r2) {
    const float w = q.w, x = q.x, y = q.y, z = q.z;
    const float xx = mul_(x, x), yy = mul_(y, y), zz = mul_(z, z);
    const float xy = mul_(x, y), xz = mul_(x, z), yz = mul_(y, z);
    const float wx = mul_(w, x), wy = mul_(w, y), wz = mul_(w, z);
    *r0 = mk3(fma_(-2.0f, add_(yy, zz), 1.0f), mul_(2.0f, sub_(xy, wz)), mul_(2.0f, add_(xz, wy)));
    *r1 = mk3(mul_(2.0f, add_(xy, wz)), fma_(-2.0f, add_(xx, zz), 1.0f), mul_(2.0f, sub_(yz, wx)));
    *r2 = mk3(mul_(2.0f, sub_(xz, wy)), mul_(2.0f, add_(yz, wx)), fma_(-2.0f, add_(xx, yy), 1.0f));
}

// Per-step constants of the packed panel pass (both halves equal).
struct PairConst {
    f2 vbx, vby, vbz;     // body-frame air velocity
    f2 wbx, wby, wbz;     // body rates
    f2 nwbx, nwby, nwbz;  // negated body rates
    f2 k19, cf, tiny, mone;
};
// Packed partial sums of one virtual lane: even panels in the low half, odd in the high half.
//   fn = sum of -f;  tq = the positive half of rb x f's products, tp = the subtracted half
struct PairAcc {
    f2 fnx, fny, fnz, tqx, tqy, tqz, tpx, tpy, tpz;
};
__device__ __forceinline__ void pair_acc_zero(PairAcc& z) {
    z.fnx = z.fny = z.fnz = z.tqx = z.tqy = z.tqz = z.tpx = z.tpy = z.tpz = 0ull;
}

// Force and torque of two panels (one pair) in the body frame, added to the partial sums.  INIT
// writes them as the sums' first terms instead of adding them to +0: the two agree unless every
// term so far is -0, and then differ only in the sign of a zero sum.
template <bool INIT = false>
__device__ __forceinline__ void fast_pair(const PairedPanels& pp, int q, const PairConst& k, float k_cf_scalar, PairAcc& acc) {
    const float4 A = pp.a[q], B = pp.b[q], C = pp.c[q];
    const float2 D = pp.d[q];
    const f2 rbx = pk(A.x, A.y), rby = pk(A.z, A.w), rbz = pk(B.x, B.y), ak = pk(B.z, B.w);
    const f2 nbx = pk(C.x, C.y), nby = pk(C.z, C.w), nbz = pk(D.x, D.y);
    // vr = v_b + wb x rb
    const f2 vx = fma2(k.wby, rbz, fma2(k.nwbz, rby, k.vbx));
    const f2 vy = fma2(k.wbz, rbx, fma2(k.nwbx, rbz, k.vby));
    const f2 vz = fma2(k.wbx, rby, fma2(k.nwby, rbx, k.vbz));
    // |vr|^2 + 1e-30: finite 1/|vr| at rest, and below half an ulp of any |vr|^2 above ~1e-23
    const f2 V2 = fma2(vz, vz, fma2(vy, vy, fma2(vx, vx, k.tiny)));
    float v2a, v2b;
    upk(V2, v2a, v2b);
    const f2 inv = pk(rsqrtf(v2a), rsqrtf(v2b));
    const f2 vn = fma2(vz, nbz, fma2(vy, nby, mul2(vx, nbx)));
    const f2 s = mul2(vn, inv);
    const f2 qd = mul2(V2, ak);
    float sa, sb;
    upk(s, sa, sb);
    // s^2 - 1 for both panels in one packed FMA; its negation rounds exactly as 1 - s^2 would
    float ua, ub;
    upk(fma2(s, s, k.mone), ua, ub);
    const f2 sq = pk(sqrtf(fmaxf(0.0f, -ua)), sqrtf(fmaxf(0.0f, -ub)));
    // cn - cf s = s (1.9 sqrt(1 - s^2) + 2 |s| - cf)
    const f2 g = fma2(k.k19, sq, pk(__fmaf_rn(2.0f, fabsf(sa), -k_cf_scalar), __fmaf_rn(2.0f, fabsf(sb), -k_cf_scalar)));
    // -f = na nb + nb_ vr with na = qd (cn - cf s), nb_ = qd cf / |vr|
    const f2 na = mul2(mul2(qd, s), g);
    const f2 nv = mul2(mul2(qd, k.cf), inv);
    const f2 nfx = fma2(na, nbx, mul2(nv, vx));
    const f2 nfy = fma2(na, nby, mul2(nv, vy));
    const f2 nfz = fma2(na, nbz, mul2(nv, vz));
    if (INIT) {  // the first pair of a virtual lane: the sums start from it, not from +0 + it
        acc.fnx = nfx; acc.fny = nfy; acc.fnz = nfz;
        acc.tqx = mul2(rbz, nfy); acc.tpx = mul2(rby, nfz);
        acc.tqy = mul2(rbx, nfz); acc.tpy = mul2(rbz, nfx);
        acc.tqz = mul2(rby, nfx); acc.tpz = mul2(rbx, nfy);
        return;
    }
    acc.fnx = add2(acc.fnx, nfx);
    acc.fny = add2(acc.fny, nfy);
    acc.fnz = add2(acc.fnz, nfz);
    // rb x f = (rbz nfy - rby nfz, rbx nfz - rbz nfx, rby nfx - rbx nfy)
    acc.tqx = fma2(rbz, nfy, acc.tqx);
    acc.tpx = fma2(rby, nfz, acc.tpx);
    acc.tqy = fma2(rbx, nfz, acc.tqy);
    acc.tpy = fma2(rbz, nfx, acc.tpy);
    acc.tqz = fma2(rby, nfx, acc.tqz);
    acc.tpz = fma2(rbx, nfy, acc.tpz);
}

// Totals of one virtual lane: force and torque, even + odd partial sums.
__device__ __forceinline__ void pair_acc_total(const PairAcc& a, float out[6]) {
    float e, o, e2, o2;
    upk(a.fnx, e, o); out[0] = -add_(e, o);
    upk(a.fny, e, o); out[1] = -add_(e, o);
    upk(a.fnz, e, o); out[2] = -add_(e, o);
    upk(a.tqx, e, o); upk(a.tpx, e2, o2); out[3] = sub_(add_(e, o), add_(e2, o2));
    upk(a.tqy, e, o); upk(a.tpy, e2, o2); out[4] = sub_(add_(e, o), add_(e2, o2));
    upk(a.tqz, e, o); upk(a.tpz, e2, o2); out[5] = sub_(add_(e, o), add_(e2, o2));
}

// Sum over the 32 virtual lanes along one xor tree, identical on every lane of the group.
// The six components (+2 zero slots) are reduced transposed: each of the first three cross-lane
// levels halves the values a lane carries (4 + 2 + 1 shuffles), the last levels are plain
// butterflies, and six shuffles broadcast the totals: 19 shuffles instead of 30.
template <int LPF>
__device__ __forceinline__ void fast_reduce(float (&acc)[32 / LPF][6], unsigned mask, int j, float out[6]) {
    constexpr int NV = 32 / LPF;
    float v[8];
#pragma unroll
    for (int c = 0; c < 6; c++) v[c] = NV == 2 ? add_(acc[0][c], acc[NV - 1][c]) : acc[0][c];
    v[6] = 0.0f;
    v[7] = 0.0f;
#pragma unroll
    for (int lv = 0; lv < 3; lv++) {
        const int m = (LPF / 2) >> lv;
        const int half = 4 >> lv;
        const bool up = (j & m) != 0;
#pragma unroll
        for (int i = 0; i < half; i++) {
            const float send = up ? v[i] : v[i + half];
            const float keep = up ? v[i + half] : v[i];
            v[i] = add_(keep, __shfl_xor_sync(mask, send, m, LPF));
        }
    }
#pragma unroll
    for (int m = LPF / 16; m >= 1; m >>= 1) v[0] = add_(v[0], __shfl_xor_sync(mask, v[0], m, LPF));
#pragma unroll
    for (int c = 0; c < 6; c++) {
        const int src = ((c >> 2) & 1) * (LPF / 2) + ((c >> 1) & 1) * (LPF / 4) + (c & 1) * (LPF / 8);
        out[c] = __shfl_sync(mask, v[0], src, LPF);
    }
}

// What the forward pass of pe_grad keeps of a step: the body-frame aerodynamic force and torque,
// and at the last step how the flight ended (1 ground, 2 other bound or horizon, 3 NaN).
struct StepOut {
    float fb[6];
    int kind;
};

template <int LPF>
__device__ __forceinline__ int fast_step(const FastConst& fc, const PairedPanels& pp, int nt, int j,
                                         unsigned mask, FlightState& st, int step, int max_steps, int smooth,
                                         float* fit, float sumw[6], StepOut* so = nullptr) {
    if (step > 0 && step % kChunk == 0) st.t = mul_((float)step, PE_DT);
    vec3 r0, r1, r2;
    fast_rows(st.q, &r0, &r1, &r2);
    const vec3 wind = fast_wind(st.pos, st.t, fc.phase, fc.gust, fc.base_x, fc.base_y);
    const vec3 va = mk3(sub_(st.vel.x, wind.x), sub_(st.vel.y, wind.y), sub_(st.vel.z, wind.z));
    // R^T va: column k of R is (r0[k], r1[k], r2[k])
    const vec3 vb = mk3(fma_(r2.x, va.z, fma_(r1.x, va.y, mul_(r0.x, va.x))),
                        fma_(r2.y, va.z, fma_(r1.y, va.y, mul_(r0.y, va.x))),
                        fma_(r2.z, va.z, fma_(r1.z, va.y, mul_(r0.z, va.x))));
    const vec3 wb = st.wb;
    PairConst k;
    k.vbx = bc(vb.x); k.vby = bc(vb.y); k.vbz = bc(vb.z);
    k.wbx = bc(wb.x); k.wby = bc(wb.y); k.wbz = bc(wb.z);
    k.nwbx = bc(-wb.x); k.nwby = bc(-wb.y); k.nwbz = bc(-wb.z);
    k.k19 = bc(PE_CN_SLOPE); k.cf = bc(fc.skin_cf); k.tiny = bc(1e-30f); k.mone = bc(-1.0f);
    constexpr int NV = 32 / LPF;
    // pass n reads pair j + LPF n, of virtual lane j + LPF (n % NV); the same count on every lane
    const int passes = ((nt + 1) / 2 + LPF - 1) / LPF;
    float acc[NV][6];
    if constexpr (NV == 2) {
        PairAcc p0, p1;
        int n = 0;
        if (passes >= 2) {
            fast_pair<true>(pp, j, k, fc.skin_cf, p0);
            fast_pair<true>(pp, j + LPF, k, fc.skin_cf, p1);
            n = 2;
        } else {
            pair_acc_zero(p0);
            pair_acc_zero(p1);
        }
        for (; n + 1 < passes; n += 2) {
            fast_pair(pp, j + LPF * n, k, fc.skin_cf, p0);
            fast_pair(pp, j + LPF * (n + 1), k, fc.skin_cf, p1);
        }
        if (n < passes) fast_pair(pp, j + LPF * n, k, fc.skin_cf, p0);
        pair_acc_total(p0, acc[0]);
        pair_acc_total(p1, acc[NV - 1]);
    } else {
        PairAcc p0;
        int n = 0;
        if (passes >= 1) {
            fast_pair<true>(pp, j, k, fc.skin_cf, p0);
            n = 1;
        } else {
            pair_acc_zero(p0);
        }
#pragma unroll 2
        for (; n < passes; n++) fast_pair(pp, j + LPF * n, k, fc.skin_cf, p0);
        pair_acc_total(p0, acc[0]);
    }
    float sum[6];
    fast_reduce<LPF>(acc, mask, j, sum);
    const vec3 Fb = mk3(sum[0], sum[1], sum[2]);
    const vec3 tb = mk3(sum[3], sum[4], sum[5]);
    if (so) {
#pragma unroll
        for (int c = 0; c < 6; c++) so->fb[c] = sum[c];
    }
    // world force for the translational update; the rotational update takes the body torque
    vec3 Fs = mk3(dot_(r0, Fb), dot_(r1, Fb), dot_(r2, Fb));
    if (sumw) {
        sumw[0] = Fs.x; sumw[1] = Fs.y; sumw[2] = Fs.z;
        sumw[3] = dot_(r0, tb); sumw[4] = dot_(r1, tb); sumw[5] = dot_(r2, tb);
    }
    Fs.z = fma_(-fc.mass, PE_GRAV, Fs.z);
    vec3 w = wb;
    const vec3 Iw = mk3(fma_(fc.I[4], w.z, fma_(fc.I[3], w.y, mul_(fc.I[0], w.x))),
                        fma_(fc.I[5], w.z, fma_(fc.I[1], w.y, mul_(fc.I[3], w.x))),
                        fma_(fc.I[2], w.z, fma_(fc.I[5], w.y, mul_(fc.I[4], w.x))));
    const vec3 gyro = mk3(fma_(w.y, Iw.z, -mul_(w.z, Iw.y)), fma_(w.z, Iw.x, -mul_(w.x, Iw.z)),
                          fma_(w.x, Iw.y, -mul_(w.y, Iw.x)));
    const vec3 tq = mk3(sub_(tb.x, gyro.x), sub_(tb.y, gyro.y), sub_(tb.z, gyro.z));
    const vec3 dw = mk3(fma_(fc.invI[2], tq.z, fma_(fc.invI[1], tq.y, mul_(fc.invI[0], tq.x))),
                        fma_(fc.invI[5], tq.z, fma_(fc.invI[4], tq.y, mul_(fc.invI[3], tq.x))),
                        fma_(fc.invI[8], tq.z, fma_(fc.invI[7], tq.y, mul_(fc.invI[6], tq.x))));
    w = mk3(fma_(dw.x, PE_DT, w.x), fma_(dw.y, PE_DT, w.y), fma_(dw.z, PE_DT, w.z));
    const float wl = sqrtf(dot_(w, w));
    if (wl > 150.f) { const float k = __fdiv_rn(150.f, wl); w = mk3(mul_(w.x, k), mul_(w.y, k), mul_(w.z, k)); }
    const float kv = mul_(fc.invmass, PE_DT);
    vec3 vel = mk3(fma_(Fs.x, kv, st.vel.x), fma_(Fs.y, kv, st.vel.y), fma_(Fs.z, kv, st.vel.z));
    const float vl = sqrtf(dot_(vel, vel));
    if (vl > 60.f) { const float k = __fdiv_rn(60.f, vl); vel = mk3(mul_(vel.x, k), mul_(vel.y, k), mul_(vel.z, k)); }
    const vec3 pos = mk3(fma_(vel.x, PE_DT, st.pos.x), fma_(vel.y, PE_DT, st.pos.y), fma_(vel.z, PE_DT, st.pos.z));
    // q += 0.5 dt q (0, w); normalize
    const quat4 q = st.q;
    const vec3 p0 = st.pos;
    const float h = mul_(0.5f, PE_DT);
    const float dqw = -fma_(q.z, w.z, fma_(q.y, w.y, mul_(q.x, w.x)));
    const float dqx = fma_(q.y, w.z, fma_(-q.z, w.y, mul_(q.w, w.x)));
    const float dqy = fma_(q.z, w.x, fma_(-q.x, w.z, mul_(q.w, w.y)));
    const float dqz = fma_(q.x, w.y, fma_(-q.y, w.x, mul_(q.w, w.z)));
    quat4 qn = mkq(fma_(h, dqw, q.w), fma_(h, dqx, q.x), fma_(h, dqy, q.y), fma_(h, dqz, q.z));
    const float il = rsqrtf(fma_(qn.z, qn.z, fma_(qn.y, qn.y, fma_(qn.x, qn.x, mul_(qn.w, qn.w)))));
    st.q = mkq(mul_(qn.w, il), mul_(qn.x, il), mul_(qn.y, il), mul_(qn.z, il));
    st.vel = vel; st.wb = w; st.pos = pos; st.t = add_(st.t, PE_DT);
    const int bad = !(pos.x == pos.x && vel.x == vel.x);
    if (pos.z <= 0.0f || bad || fabsf(pos.y) > 300.f || pos.x < -50.f) {
        *fit = bad ? -10.0f : pos.x;
        if (smooth && !bad && pos.z <= 0.0f) {  // the z = 0 crossing between the last two states
            const float a = __fdiv_rn(p0.z, sub_(p0.z, pos.z));
            *fit = fma_(sub_(pos.x, p0.x), a, p0.x);
        }
        if (so) so->kind = bad ? 3 : (pos.z <= 0.0f ? 1 : 2);
        return 1;
    } else if (step == max_steps - 1) {
        *fit = pos.x;
        if (so) so->kind = 2;
        return 1;
    }
    return 0;
}

template <int LPF>
__device__ __forceinline__ unsigned fast_mask(int lane) {
    return LPF == 32 ? 0xffffffffu : (0xffffu << (lane & 16));
}

// Record slot of step `step` in the reference's gpu_sim (src/sim.cu:115-121): every 600-step launch
// restarts its index at step0 / rec_every and advances it at each multiple of rec_every, so when
// rec_every does not divide 600 a launch's first record overwrites the previous launch's last.
__device__ __forceinline__ int rec_slot(int step, int every) {
    const int s0 = step - step % kChunk;
    const int before = s0 == 0 ? 0 : (s0 - 1) / every + 1;  // multiples of `every` in [0, s0)
    return s0 / every + (step / every + 1 - before) - 1;
}
__device__ __forceinline__ void rec_put(const FlightArgs& a, int flight, int step, const FlightState& st,
                                        float alive) {
    const int i = rec_slot(step, a.rec_every);
    if (i >= a.rec_cap) return;
    float4* r = reinterpret_cast<float4*>(a.rec + ((size_t)flight * a.rec_cap + i) * 8);
    r[0] = make_float4(st.pos.x, st.pos.y, st.pos.z, st.q.w);
    r[1] = make_float4(st.q.x, st.q.y, st.q.z, alive);
}
// The frozen pose of a finished flight at every record step after `from` (-1: from step 0; lanes
// share the steps).
__device__ __forceinline__ void rec_fill(const FlightArgs& a, int flight, int from, const FlightState& st, int j,
                                         int lanes) {
    const int first = from < 0 ? 0 : (from / a.rec_every + 1) * a.rec_every;
    for (int m = first + j * a.rec_every; m < kMaxSteps; m += lanes * a.rec_every) rec_put(a, flight, m, st, 0.f);
}

// CAP = 1 caps registers at 96 (launch bounds of 5 blocks x 128 threads), CAP = 2 at 128 (4 blocks
// x 128 threads): more flights reside per SM; spilled values go to L1-resident local memory.
// CAP = 3 launches one-warp blocks, 11 per SM (registers <= 184, no spills): at 16 lanes that is
// all the 2-flight slots shared memory holds (11 x (2 x 9,856 B + 1 KB reserved) of 228 KB), one
// warp more per SM than the uncapped kernel's 198 registers leave room for.
// REC = true adds the reference's pose recording and launch grid (pe_sim only).
// GRAD = true is pe_grad's forward pass: every flight from its set-up record (FlightArgs.grad_setup),
// smoothed distances, and per flight its checkpoints, every step's body force and torque and how it
// ended (FlightArgs.grad_*); one launch over all flights.
template <int LPF, int CAP, bool REC = false, bool GRAD = false>
__global__ void __launch_bounds__(CAP == 3 ? 32 : (CAP ? 128 : 256), CAP == 1 ? 5 : (CAP == 2 ? 4 : (CAP == 3 ? 11 : 1)))
    k_flight_fast(FlightArgs a) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int j = lane % LPF;
    const int slot = threadIdx.x / LPF;
    const PairedPanels pp = paired_view<LPF>((char*)smem + (size_t)slot * paired_bytes<LPF>());
    const unsigned mask = fast_mask<LPF>(lane);
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
        FastConst fc;
        vec3 cg;
        float air_rho, wp, wr;
        FlightState st;
        if (GRAD) {  // the gradient model's set-up of this flight
            const float* r = a.grad_setup + (size_t)flight * kGradSetupFloats;
            fc.mass = r[0]; fc.invmass = r[1];
            for (int c = 0; c < 6; c++) fc.I[c] = r[2 + c];
            for (int c = 0; c < 9; c++) fc.invI[c] = r[8 + c];
            fc.skin_cf = r[17]; fc.phase = r[18]; fc.gust = r[19]; fc.base_x = r[20]; fc.base_y = r[21];
            cg = mk3(r[22], r[23], r[24]);
            air_rho = r[25]; wp = r[26]; wr = r[27];
            st = *reinterpret_cast<const FlightState*>(r + 32);
            if (nt <= 0) {
                if (j == 0) { a.dist[flight] = -100.0f; a.steps[flight] = 0; a.grad_kind[flight] = 0; }
                continue;
            }
        } else {
            MassProps pmp;
            Scenario sc;
            fast_setup(a, p, s, &fc, &cg, &air_rho, &wp, &wr, &pmp, &sc);
            if (a.step_begin == 0) {
                if (REC || nt > 0) release(sc, pmp, cg, &st);
                if (REC && a.spread > 0.f) {  // showcase launch grid, src/sim.cu:72-79
                    const int cols = 25;
                    st.pos.x = -(float)(p / cols) * a.spread * 1.4f;
                    st.pos.y = (float)((p % cols) - cols / 2) * a.spread;
                    st.pos.z = st.pos.z + 0.25f * sinf((float)p * 12.9898f);
                }
                if (nt <= 0) {
                    if (j == 0) { a.dist[flight] = -100.0f; a.steps[flight] = 0; }
                    if (REC && a.rec) rec_fill(a, flight, -1, st, j, LPF);
                    continue;
                }
            } else {
                st = a.state[flight];
            }
        }
        float* ck = nullptr;
        float* fsum = nullptr;
        if (GRAD) {
            ck = a.grad_ck + (size_t)flight * a.grad_nck * 16;
            fsum = a.grad_fsum ? a.grad_fsum + (size_t)flight * a.max_steps * 8 : nullptr;
            if (j == 0) *reinterpret_cast<FlightState*>(ck) = st;  // the release state
        }
        __syncwarp(mask);
        fast_stage<LPF>(a, p, nt, j, cg, air_rho, wp, wr, pp);
        __syncwarp(mask);
        const int end = min(a.step_end, a.max_steps);
        int step = st.step, done = 0;
        float fit = 0.0f;
        StepOut so;
        so.kind = 0;
        int to_ck = GRAD ? a.grad_K : 0, ck_i = 0;  // steps to the next checkpoint, its index
        for (; step < end; step++) {
            if (REC && a.rec && j == 0 && step % a.rec_every == 0) rec_put(a, flight, step, st, 1.f);
            done = fast_step<LPF>(fc, pp, nt, j, mask, st, step, a.max_steps, GRAD ? 1 : a.smooth, &fit, nullptr,
                                  GRAD ? &so : nullptr);
            if (GRAD && j == 0) {
                if (fsum) {
                    float4* d4 = reinterpret_cast<float4*>(fsum + (size_t)step * 8);
                    d4[0] = make_float4(so.fb[0], so.fb[1], so.fb[2], so.fb[3]);
                    d4[1] = make_float4(so.fb[4], so.fb[5], 0.0f, 0.0f);
                }
            }
            if (GRAD && --to_ck == 0) {  // after step + 1 = (ck_i + 1) * K steps
                to_ck = a.grad_K;
                ++ck_i;
                if (!done && j == 0) {
                    FlightState c = st;  // as the next step starts: the clock restarts every 600 steps
                    if ((step + 1) % kChunk == 0) c.t = mul_((float)(step + 1), PE_DT);
                    *reinterpret_cast<FlightState*>(ck + (size_t)ck_i * 16) = c;
                }
            }
            if (done) break;
        }
        if (done) {
            if (GRAD && j == 0) a.grad_kind[flight] = so.kind;
            if (j == 0) { a.dist[flight] = fit; a.steps[flight] = step + 1; }
            if (REC && a.rec) {
                __syncwarp(mask);  // lane 0's alive frames precede the frozen ones that may share a slot
                rec_fill(a, flight, step, st, j, LPF);
            }
        } else if (j == 0 && a.active_out) {
            st.step = step;
            a.state[flight] = st;
            int k = atomicAdd(a.n_active_out, 1);
            a.active_out[k] = flight;
        }
    }
}

template <int LPF>
__global__ void __launch_bounds__(256) k_debug_step_fast(FlightArgs a, const FlightState* state_in,
                                                         FlightState* state_out, float* FT, int* done_out,
                                                         float* fit_out, int step) {
    extern __shared__ float4 smem[];
    const int lane = threadIdx.x & 31;
    const int j = lane % LPF;
    const int slot = threadIdx.x / LPF;
    const PairedPanels pp = paired_view<LPF>((char*)smem + (size_t)slot * paired_bytes<LPF>());
    const unsigned mask = fast_mask<LPF>(lane);
    const int flight = blockIdx.x * (blockDim.x / LPF) + slot;
    if (flight >= a.n_flights) return;
    const int p = flight / a.nseeds, s = flight - p * a.nseeds;
    const int nt = a.plane_nt[p];
    FastConst fc;
    vec3 cg;
    float air_rho, wp, wr;
    fast_setup(a, p, s, &fc, &cg, &air_rho, &wp, &wr, nullptr, nullptr);
    fast_stage<LPF>(a, p, nt, j, cg, air_rho, wp, wr, pp);
    __syncwarp(mask);
    FlightState st = state_in[flight];
    float fit = 0.0f, sumw[6];
    int done = fast_step<LPF>(fc, pp, nt, j, mask, st, step, a.max_steps, 0, &fit, sumw);
    if (j == 0) {
        state_out[flight] = st;
        for (int c = 0; c < 6; c++) FT[flight * 6 + c] = sumw[c];
        done_out[flight] = done;
        fit_out[flight] = fit;
    }
}

template <int LPF>
static const void* fast_fn_lanes(int cap) {
    switch (cap) {
        case 1: return (const void*)&k_flight_fast<LPF, 1>;
        case 2: return (const void*)&k_flight_fast<LPF, 2>;
        case 3: return (const void*)&k_flight_fast<LPF, 3>;
        default: return (const void*)&k_flight_fast<LPF, 0>;
    }
}
static const void* fast_fn(const FlightShape& sh) {
    return sh.lanes == 16 ? fast_fn_lanes<16>(sh.cap) : fast_fn_lanes<32>(sh.cap);
}
template <int LPF>
static void launch_lanes(const FlightArgs& a, int cap, int grid, int threads, size_t smem, cudaStream_t s) {
    switch (cap) {
        case 1: k_flight_fast<LPF, 1><<<grid, threads, smem, s>>>(a); break;
        case 2: k_flight_fast<LPF, 2><<<grid, threads, smem, s>>>(a); break;
        case 3: k_flight_fast<LPF, 3><<<grid, threads, smem, s>>>(a); break;
        default: k_flight_fast<LPF, 0><<<grid, threads, smem, s>>>(a);
    }
}

size_t flight_fast_smem_bytes(const FlightShape& sh) {
    return (size_t)(sh.warps * 32 / sh.lanes) * (sh.lanes == 16 ? paired_bytes<16>() : paired_bytes<32>());
}

int flight_fast_blocks_per_sm(const FlightShape& sh) {
    const void* fn = fast_fn(sh);
    size_t smem = flight_fast_smem_bytes(sh);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, sh.warps * 32, smem) != cudaSuccess) return 0;
    return nb;
}

cudaError_t launch_flight_fast(const FlightArgs& a, const FlightShape& sh, int grid, cudaStream_t s) {
    size_t smem = flight_fast_smem_bytes(sh);
    const void* fn = fast_fn(sh);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if ((sh.cap && sh.warps > 4) || (sh.cap == 3 && sh.warps != 1) || sh.cap < 0 || sh.cap > 3)
        return cudaErrorInvalidValue;
    const int threads = sh.warps * 32;
    if (a.rec || a.spread > 0.f) {  // recording and the launch grid run in the default shape only
        if (sh.lanes != 16 || sh.cap) return cudaErrorInvalidValue;
        e = cudaFuncSetAttribute((const void*)&k_flight_fast<16, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        k_flight_fast<16, 0, true><<<grid, threads, smem, s>>>(a);
    } else if (sh.lanes == 16) {
        launch_lanes<16>(a, sh.cap, grid, threads, smem, s);
    } else if (sh.lanes == 32) {
        launch_lanes<32>(a, sh.cap, grid, threads, smem, s);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t grad_forward_configure(int bps[2]) {
    const void* fn[2] = {(const void*)&k_flight_fast<32, 0, false, true>, (const void*)&k_flight_fast<16, 3, false, true>};
    const int threads[2] = {128, 32};
    const size_t smem[2] = {4 * paired_bytes<32>(), 2 * paired_bytes<16>()};
    for (int i = 0; i < 2; i++) {
        cudaError_t e = cudaFuncSetAttribute(fn[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[i]);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps[i], fn[i], threads[i], smem[i]);
        if (e != cudaSuccess) return e;
        if (bps[i] <= 0) bps[i] = 1;
    }
    return cudaSuccess;
}

cudaError_t launch_grad_forward(const FlightArgs& a, int nsm, const int bps[2], cudaStream_t s) {
    if (!a.grad_setup || !a.grad_ck || !a.grad_kind || a.grad_K < 1 || a.step_begin != 0 ||
        a.step_end < a.max_steps || a.active_in || a.active_out)
        return cudaErrorInvalidValue;
    const bool small = (long long)a.n_flights <= 192LL * nsm;
    const int threads = small ? 128 : 32;
    const size_t smem = small ? 4 * paired_bytes<32>() : 2 * paired_bytes<16>();
    const int grid = bps[small ? 0 : 1] * nsm;
    if (small)
        k_flight_fast<32, 0, false, true><<<grid, threads, smem, s>>>(a);
    else
        k_flight_fast<16, 3, false, true><<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_debug_step_fast(const FlightArgs& a, const FlightState* state_in, FlightState* state_out,
                                   float* FT, int* done, float* fit, int step, int lanes, cudaStream_t s) {
    const int threads = 128;
    const int per_block = threads / lanes;
    const int grid = (a.n_flights + per_block - 1) / per_block;
    const size_t smem = (size_t)per_block * (lanes == 16 ? paired_bytes<16>() : paired_bytes<32>());
    if (lanes == 16) {
        cudaFuncSetAttribute((const void*)&k_debug_step_fast<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_debug_step_fast<16><<<grid, threads, smem, s>>>(a, state_in, state_out, FT, done, fit, step);
    } else {
        cudaFuncSetAttribute((const void*)&k_debug_step_fast<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_debug_step_fast<32><<<grid, threads, smem, s>>>(a, state_in, state_out, FT, done, fit, step);
    }
    return cudaGetLastError();
}

}  // namespace pe
