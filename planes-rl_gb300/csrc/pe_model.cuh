// pe_model.cuh -- device-side physics of the planes-rl fitness path (GB300 / sm_103a).
//
// This header holds the per-plane and per-flight model: genome layout, the implicit mirrored
// mesh (vertex and triangle of any index, no stored index buffer), mass properties, the
// scenario draw, print variation, the gust field and the release.  Each function computes the
// same quantity with the same operand order as the reference (citations are to files of the
// reference project), and the translation units that include it are compiled with
// -use_fast_math as the reference is (Makefile:3), so sinf/cosf/tanf/sqrtf/division lower to
// the same hardware approximations.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pe {

// ------------------------------------------------------------------ sizes
constexpr int kGenomeN = 35;     // floats per genome, src/common.h:60
constexpr int kMpN = 20;         // floats per MassProps, src/common.h:117-122
constexpr int kScenN = 25;       // floats per ScenarioDesc, src/common.h:377-387
constexpr int kCH = 5, kSP = 8;  // src/common.h:106-107
constexpr int kWingV = (2 * kSP + 1) * (kCH + 1);  // 102
constexpr int kWingT = 2 * kSP * kCH * 2;          // 160
// Triangle/vertex counts are fixed by the topology (deck_gap, fin_layout):
//   nt = 174 + 2*fins (+164 biplane) <= 344,  nv = 119 + 4*fins (+110 biplane) <= 241.
constexpr int kNtMax = 344;
constexpr int kNvMax = 241;
constexpr int kChunk = 600;      // the reference's launch length; its clock restarts there
constexpr int kMaxSteps = 7200;  // SIM_MAX_STEPS, src/common.h:471
#define PE_DT (1.0f / 600.0f)    // SIM_DT
#define PE_CN_SLOPE 1.9f
#define PE_GRAV 9.81f
#define PE_SHELL_RHO (1240.0f * 0.00045f)
#define PE_WALL 0.00045f
#define PE_PRINT_LIMIT (0.250f - 0.00045f)

// genome gene indices (src/common.h:61-97)
enum Gene {
    G_SPAN, G_CHORD, G_TAPER, G_SWEEP, G_DIH_IN, G_DIH_OUT, G_KINK, G_CAMBER1, G_CAMBER2,
    G_WASHOUT, G_ELEVATOR, G_NOSE, G_KEEL, G_DECK_GAP, G_DECK_SCALE, G_BODY, G_FIN_H,
    G_FIN_CHORD, G_FIN_SWEEP, G_TAIL_SPAN, G_TAIL_CHORD, G_TAIL_ANGLE, G_LE_B1, G_LE_B2,
    G_CHORD_B1, G_CHORD_B2, G_FIN_LAYOUT, G_FIN_CANT, G_FIN_TAPER, G_FIN_SPAN_POS,
    G_TAIL_SWEEP, G_TAIL_TAPER, G_TAIL_DIH, G_TIP_ROUND, G_CENTER_CHORD
};

// scenario field indices (src/common.h:377-387)
enum Scen {
    S_SPEED, S_PITCH, S_YAW, S_ROLL, S_HEIGHT, S_ROLL_RATE, S_PITCH_RATE, S_YAW_RATE, S_AIR_RHO,
    S_SKIN_CF, S_GUST, S_BASE_X, S_BASE_Y, S_FORCE_PITCH, S_FORCE_YAW, S_GRIP_X, S_GRIP_Y,
    S_GRIP_Z, S_MATERIAL, S_INFILL, S_BIAS_X, S_BIAS_Y, S_BIAS_Z, S_WARP_PITCH, S_WARP_ROLL
};

// ------------------------------------------------------------------ vec / quat
struct vec3 { float x, y, z; };
struct quat4 { float w, x, y, z; };

__device__ __forceinline__ vec3 mk3(float x, float y, float z) { vec3 a; a.x = x; a.y = y; a.z = z; return a; }
__device__ __forceinline__ vec3 vadd(vec3 a, vec3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ vec3 vsub(vec3 a, vec3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ vec3 vscl(vec3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float vdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ vec3 vcross(vec3 a, vec3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float vlen(vec3 a) { return sqrtf(vdot(a, a)); }
__device__ __forceinline__ vec3 vnorm(vec3 a) {
    float l = vlen(a);
    return l > 1e-12f ? vscl(a, 1.0f / l) : mk3(0, 0, 1);
}
__device__ __forceinline__ quat4 mkq(float w, float x, float y, float z) { quat4 q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }
__device__ __forceinline__ quat4 qmul(quat4 a, quat4 b) {
    return mkq(a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
               a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
               a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
               a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w);
}
__device__ __forceinline__ quat4 qnormalize(quat4 q) {
    float l = sqrtf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    float il = 1.0f / l;
    return mkq(q.w * il, q.x * il, q.y * il, q.z * il);
}
// body->world rotation rows (src/common.h:38-43)
__device__ __forceinline__ void qrows(quat4 q, vec3* r0, vec3* r1, vec3* r2) {
    float w = q.w, x = q.x, y = q.y, z = q.z;
    *r0 = mk3(1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y));
    *r1 = mk3(2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x));
    *r2 = mk3(2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y));
}
__device__ __forceinline__ vec3 qrot(quat4 q, vec3 v) {
    vec3 r0, r1, r2; qrows(q, &r0, &r1, &r2);
    return mk3(vdot(r0, v), vdot(r1, v), vdot(r2, v));
}
__device__ __forceinline__ vec3 qrot_inv(quat4 q, vec3 v) {
    vec3 r0, r1, r2; qrows(q, &r0, &r1, &r2);
    return mk3(r0.x * v.x + r1.x * v.y + r2.x * v.z,
               r0.y * v.x + r1.y * v.y + r2.y * v.z,
               r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
__device__ __forceinline__ quat4 qaxis(vec3 axis, float ang) {
    float s = sinf(ang * 0.5f); vec3 a = vnorm(axis);
    return mkq(cosf(ang * 0.5f), a.x * s, a.y * s, a.z * s);
}

// ------------------------------------------------------------------ mesher
// One genome, read through a pointer to its 35 floats (shared or global memory).
struct GenomeRef {
    const float* g;
    __device__ __forceinline__ float operator[](int i) const { return g[i]; }
};

// src/common.h:124-129
__device__ __forceinline__ float camber_z(GenomeRef g, float xc) {
    float te = g[G_ELEVATOR] * 0.22f;
    float u = xc, v = 1.0f - u;
    return 3 * v * v * u * g[G_CAMBER1] + 3 * v * u * u * g[G_CAMBER2] + u * u * u * te;
}
// src/common.h:132-141
__device__ __forceinline__ void span_yz(GenomeRef g, float t, float* y, float* z) {
    float half = g[G_SPAN] * 0.5f;
    float b = g[G_BODY] * half, k = g[G_KINK] * half;
    if (k < b) k = b;
    float yy = 0, zz = 0, seg;
    seg = fminf(t, b); yy += seg;
    seg = fminf(t, k) - b;
    if (seg > 0) { yy += seg * cosf(g[G_DIH_IN]); zz += seg * sinf(g[G_DIH_IN]); }
    seg = t - k;
    if (seg > 0) { yy += seg * cosf(g[G_DIH_OUT]); zz += seg * sinf(g[G_DIH_OUT]); }
    *y = yy; *z = zz;
}
// src/common.h:144-172
static __device__ __noinline__ vec3 wing_pt(GenomeRef g, float u, float xc, float zoff, float scale) {
    float half = g[G_SPAN] * 0.5f * scale;
    float t = fabsf(u) * half;
    float y, z; span_yz(g, t, &y, &z);
    float tf = fabsf(u);
    float v = 1.0f - tf;
    float cr = 1.0f + g[G_CENTER_CHORD];
    float ct = g[G_TAPER];
    float c1 = 1.0f + g[G_CHORD_B1], c2 = ct + g[G_CHORD_B2];
    float ratio = v * v * v * cr + 3 * v * v * tf * c1 + 3 * v * tf * tf * c2 + tf * tf * tf * ct;
    float ellipse = sqrtf(fmaxf(0.08f, 1.0f - 0.92f * tf * tf));
    ratio *= 1.0f - g[G_TIP_ROUND] + g[G_TIP_ROUND] * ellipse;
    ratio = fmaxf(0.035f, fminf(1.9f, ratio));
    float c = g[G_CHORD] * scale * ratio;
    float xr = 0.5f * g[G_CHORD] * scale * cr;
    float xt = 0.5f * g[G_CHORD] * scale - tanf(g[G_SWEEP]) * half;
    float xb1 = xr + g[G_LE_B1] * g[G_CHORD] * scale;
    float xb2 = xt + g[G_LE_B2] * g[G_CHORD] * scale;
    float x_le = v * v * v * xr + 3 * v * v * tf * xb1 + 3 * v * tf * tf * xb2 + tf * tf * tf * xt;
    float x = x_le - xc * c;
    float zc = z * scale + camber_z(g, xc) * c;
    float x_c4 = x_le - 0.25f * c;
    float tw = g[G_WASHOUT] * tf;
    zc += tw * (x - x_c4);
    return mk3(x, (u < 0 ? -y : y), zc + zoff);
}

// Topology of one genome: fins and decks decide every index range of the mesh.
struct Topo {
    int nfins;      // 1..3
    int fin_mode;   // 0 center, 1 twin, 2 triple, 3 outboard (src/common.h:240-254)
    int bi;         // biplane deck (src/common.h:261)
    int nv, nt;
};
__device__ __forceinline__ Topo topology(GenomeRef g) {
    Topo t;
    float lay = g[G_FIN_LAYOUT];
    t.fin_mode = lay < 0.25f ? 0 : (lay < 0.50f ? 1 : (lay < 0.75f ? 2 : 3));
    t.nfins = t.fin_mode == 2 ? 3 : (t.fin_mode == 0 ? 1 : 2);
    t.bi = g[G_DECK_GAP] > 0.02f ? 1 : 0;
    t.nv = kWingV + 9 + 4 * t.nfins + 8 + (t.bi ? kWingV + 8 : 0);
    t.nt = kWingT + 8 + 2 * t.nfins + 6 + (t.bi ? kWingT + 4 : 0);
    return t;
}

// Chordwise stations j / CH and j / 3 of the wing grid and keel.  The reference's loops over
// these stations have constant trip counts, so its compiler folds the quotients to correctly
// rounded constants; 1 selects that (default), 0 the run-time fast-math quotient.
static __constant__ int c_station_ieee = 1;
__device__ __forceinline__ float station(int j, int n) {
    return c_station_ieee ? __fdiv_rn((float)j, (float)n) : (float)j / n;
}

// Vertex `idx` of the mesh that build_mesh (src/common.h:257-292) would emit at that index.
static __device__ __noinline__ vec3 mesh_vertex(GenomeRef g, const Topo& tp, int idx) {
    if (idx < kWingV) {  // main wing grid, emit_wing(zoff=0, scale=1)
        int i = idx / (kCH + 1), j = idx % (kCH + 1);
        float u = (float)(i - kSP) / kSP;
        float xc = station(j, kCH);
        return wing_pt(g, u, xc, 0, 1.0f);
    }
    idx -= kWingV;
    float hs = 0.5f * g[G_SPAN] * g[G_TAIL_SPAN];
    float z0 = camber_z(g, 0.82f) * g[G_CHORD];
    if (idx < 9) {  // horizontal tail 3x3 grid (src/common.h:215-236)
        int i = idx / 3, j = idx % 3;
        float hc = g[G_CHORD] * g[G_TAIL_CHORD];
        float x0 = -0.32f * g[G_CHORD];
        float u = (float)(i - 1), au = fabsf(u);
        float tc = hc * (1.0f + (g[G_TAIL_TAPER] - 1.0f) * au);
        float xle = x0 - g[G_TAIL_SWEEP] * hc * au;
        float xc = 0.5f * j;
        float x = xle - xc * tc;
        float z = z0 + g[G_TAIL_ANGLE] * (x - xle) + au * hs * sinf(g[G_TAIL_DIH]);
        return mk3(x, u * hs * cosf(g[G_TAIL_DIH]), z);
    }
    idx -= 9;
    if (idx < 4 * tp.nfins) {  // fins, emit_one_fin (src/common.h:197-213) in layout order
        int f = idx >> 2, c = idx & 3;
        float y0, zb; int side;
        if (tp.fin_mode == 3) {
            float yo = hs * 0.94f * cosf(g[G_TAIL_DIH]);
            float zo = z0 + hs * 0.94f * sinf(g[G_TAIL_DIH]);
            side = f == 0 ? -1 : 1; y0 = f == 0 ? -yo : yo; zb = zo;
        } else {
            int k = tp.fin_mode == 1 ? f + 1 : f;  // twin: fins 1,2 of the triple list
            if (k == 0) { side = 0; y0 = 0; zb = z0; }
            else {
                float yp = hs * g[G_FIN_SPAN_POS] * cosf(g[G_TAIL_DIH]);
                float zp = z0 + hs * g[G_FIN_SPAN_POS] * sinf(g[G_TAIL_DIH]);
                side = k == 1 ? -1 : 1; y0 = k == 1 ? -yp : yp; zb = zp;
            }
        }
        float fc = g[G_CHORD] * g[G_FIN_CHORD];
        float xr = -0.32f * g[G_CHORD] - g[G_TAIL_CHORD] * g[G_CHORD] * 0.82f;
        if (c < 2) return mk3(c == 0 ? xr + 0.5f * fc : xr - 0.5f * fc, y0, zb);
        float sweep = fc * g[G_FIN_SWEEP];
        float tipc = fc * g[G_FIN_TAPER];
        float cant = side == 0 ? 0.0f : g[G_FIN_CANT];
        float ya = y0 + side * sinf(cant) * g[G_FIN_H];
        float za = zb + cosf(cant) * g[G_FIN_H];
        return mk3(c == 2 ? xr - sweep + 0.5f * tipc : xr - sweep - 0.5f * tipc, ya, za);
    }
    idx -= 4 * tp.nfins;
    if (tp.bi) {
        if (idx < kWingV) {  // upper deck, emit_wing(zoff=deck_gap, scale=deck_scale)
            int i = idx / (kCH + 1), j = idx % (kCH + 1);
            float u = (float)(i - kSP) / kSP;
            float xc = station(j, kCH);
            return wing_pt(g, u, xc, g[G_DECK_GAP], g[G_DECK_SCALE]);
        }
        idx -= kWingV;
    }
    if (idx < 8) {  // keel sheet (src/common.h:264-277)
        int j = idx >> 1;
        float xc = station(j, 3);
        vec3 top = wing_pt(g, 0, xc, 0, 1.0f);
        if ((idx & 1) == 0) return top;
        return mk3(top.x, 0, top.z - g[G_KEEL] * (0.35f + 0.65f * xc));
    }
    idx -= 8;
    // biplane struts (src/common.h:279-290)
    int s = (idx >> 2) == 0 ? -1 : 1, c = idx & 3;
    float u = s * g[G_KINK];
    if (c == 0) return wing_pt(g, u, 0.25f, 0, 1.0f);
    if (c == 1) return wing_pt(g, u, 0.55f, 0, 1.0f);
    return wing_pt(g, u * 1.0f, c == 2 ? 0.25f : 0.55f, g[G_DECK_GAP], g[G_DECK_SCALE]);
}

// Vertex indices of triangle `t`, in build_mesh's emission order.
__device__ __forceinline__ void mesh_tri(const Topo& tp, int t, int* ia, int* ib, int* ic) {
    int vb = 0;
    if (t < kWingT) goto grid;
    t -= kWingT; vb = kWingV;
    if (t < 8) {  // tail grid 2x2 quads
        int q = t >> 1, i = q >> 1, j = q & 1;
        int a = vb + i * 3 + j, b = a + 3;
        if (t & 1) { *ia = b; *ib = b + 1; *ic = a + 1; } else { *ia = a; *ib = b; *ic = a + 1; }
        return;
    }
    t -= 8; vb += 9;
    if (t < 2 * tp.nfins) {
        int base = vb + 4 * (t >> 1);
        if (t & 1) { *ia = base + 1; *ib = base + 3; *ic = base + 2; } else { *ia = base; *ib = base + 1; *ic = base + 2; }
        return;
    }
    t -= 2 * tp.nfins; vb += 4 * tp.nfins;
    if (tp.bi) {
        if (t < kWingT) goto grid;
        t -= kWingT; vb += kWingV;
    }
    if (t < 6) {  // keel
        int a = vb + (t >> 1) * 2;
        if (t & 1) { *ia = a + 1; *ib = a + 3; *ic = a + 2; } else { *ia = a; *ib = a + 1; *ic = a + 2; }
        return;
    }
    t -= 6; vb += 8;
    {   // struts
        int base = vb + 4 * (t >> 1);
        if (t & 1) { *ia = base + 1; *ib = base + 3; *ic = base + 2; } else { *ia = base; *ib = base + 1; *ic = base + 2; }
        return;
    }
grid: {
        int q = t >> 1, i = q / kCH, j = q % kCH;
        int a = vb + i * (kCH + 1) + j, b = a + kCH + 1;
        if (t & 1) { *ia = b; *ib = b + 1; *ic = a + 1; } else { *ia = a; *ib = b; *ic = a + 1; }
    }
}

// ------------------------------------------------------------------ mass properties
// MassProps layout: mass, invmass, com[3], I[6] (xx yy zz xy xz yz), invI[9].
struct MassProps {
    float mass, invmass;
    vec3 com;
    float I[6];
    float invI[9];
};

// src/common.h:311-365 by one warp.  The lanes compute every triangle's terms in parallel into
// shared memory (T: kMpTerms x kNtMax floats, term k of triangle i at T[k * kNtMax + i]); lane 0
// then adds them in emission order with the same expressions as a one-thread loop, so the sums
// round exactly as the reference's serial loop does.  Two passes, as in the reference: the centre
// of mass first, then the inertia about it.  The 3x3 inverse that the flight never reads (the
// print-varied inverse replaces it) is taken in FP64.  Called by all 32 lanes; *mp on lane 0.
constexpr int kMpTerms = 15;
static __device__ __noinline__ void mass_props(GenomeRef g, const vec3* V, const Topo& tp, int lane, float* T,
                                               float* s_c, MassProps* mp) {
    for (int i = lane; i < tp.nt; i += 32) {
        int ia, ib, ic; mesh_tri(tp, i, &ia, &ib, &ic);
        vec3 a = V[ia], b = V[ib], d = V[ic];
        float A = 0.5f * vlen(vcross(vsub(b, a), vsub(d, a)));
        float mi = A * PE_SHELL_RHO;
        vec3 ct = vscl(vadd(vadd(a, b), d), 1.0f / 3);
        T[i] = mi; T[kNtMax + i] = ct.x; T[2 * kNtMax + i] = ct.y; T[3 * kNtMax + i] = ct.z;
    }
    __syncwarp();
    float m = 0, mn = 0;
    vec3 c = mk3(0, 0, 0), np = mk3(0, 0, 0);
    if (lane == 0) {
        for (int i = 0; i < tp.nt; i++) {
            float mi = T[i];
            vec3 ct = mk3(T[kNtMax + i], T[2 * kNtMax + i], T[3 * kNtMax + i]);
            m += mi; c = vadd(c, vscl(ct, mi));
        }
        float shell_m = m;
        np = mk3(0.5f * g[G_CHORD], 0, 0);
        mn = g[G_NOSE] * shell_m;
        m += mn; c = vadd(c, vscl(np, mn));
        c = vscl(c, 1.0f / m);
        s_c[0] = c.x; s_c[1] = c.y; s_c[2] = c.z;
    }
    __syncwarp();
    c = mk3(s_c[0], s_c[1], s_c[2]);
    for (int i = lane; i < tp.nt; i += 32) {
        int ia, ib, ic; mesh_tri(tp, i, &ia, &ib, &ic);
        vec3 a = V[ia], b = V[ib], d = V[ic];
        float A = 0.5f * vlen(vcross(vsub(b, a), vsub(d, a)));
        float mi = A * PE_SHELL_RHO;
        vec3 ra = vsub(a, c), rb = vsub(b, c), rd = vsub(d, c);
        float exx = (ra.x * ra.x + rb.x * rb.x + rd.x * rd.x + ra.x * rb.x + ra.x * rd.x + rb.x * rd.x) / 6.0f;
        float eyy = (ra.y * ra.y + rb.y * rb.y + rd.y * rd.y + ra.y * rb.y + ra.y * rd.y + rb.y * rd.y) / 6.0f;
        float ezz = (ra.z * ra.z + rb.z * rb.z + rd.z * rd.z + ra.z * rb.z + ra.z * rd.z + rb.z * rd.z) / 6.0f;
        float exy = (2 * (ra.x * ra.y + rb.x * rb.y + rd.x * rd.y) +
                     ra.x * rb.y + rb.x * ra.y + ra.x * rd.y + rd.x * ra.y + rb.x * rd.y + rd.x * rb.y) / 12.0f;
        float exz = (2 * (ra.x * ra.z + rb.x * rb.z + rd.x * rd.z) +
                     ra.x * rb.z + rb.x * ra.z + ra.x * rd.z + rd.x * ra.z + rb.x * rd.z + rd.x * rb.z) / 12.0f;
        float eyz = (2 * (ra.y * ra.z + rb.y * rb.z + rd.y * rd.z) +
                     ra.y * rb.z + rb.y * ra.z + ra.y * rd.z + rd.y * ra.z + rb.y * rd.z + rd.y * rb.z) / 12.0f;
        vec3 nn = vnorm(vcross(vsub(b, a), vsub(d, a)));
        float th = mi * PE_WALL * PE_WALL / 12.0f;
        float* t = T + i;
        t[0] = mi; t[kNtMax] = eyy + ezz; t[2 * kNtMax] = exx + ezz; t[3 * kNtMax] = exx + eyy;
        t[4 * kNtMax] = exy; t[5 * kNtMax] = exz; t[6 * kNtMax] = eyz;
        t[7 * kNtMax] = th; t[8 * kNtMax] = 1.0f - nn.x * nn.x; t[9 * kNtMax] = 1.0f - nn.y * nn.y;
        t[10 * kNtMax] = 1.0f - nn.z * nn.z; t[11 * kNtMax] = th * nn.x; t[12 * kNtMax] = th * nn.y;
        t[13 * kNtMax] = nn.y; t[14 * kNtMax] = nn.z;
    }
    __syncwarp();
    if (lane != 0) return;
    float I[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < tp.nt; i++) {
        const float* t = T + i;
        float mi = t[0];
        I[0] += mi * t[kNtMax]; I[1] += mi * t[2 * kNtMax]; I[2] += mi * t[3 * kNtMax];
        I[3] -= mi * t[4 * kNtMax]; I[4] -= mi * t[5 * kNtMax]; I[5] -= mi * t[6 * kNtMax];
        float th = t[7 * kNtMax];
        I[0] += th * t[8 * kNtMax]; I[1] += th * t[9 * kNtMax]; I[2] += th * t[10 * kNtMax];
        I[3] -= t[11 * kNtMax] * t[13 * kNtMax]; I[4] -= t[11 * kNtMax] * t[14 * kNtMax];
        I[5] -= t[12 * kNtMax] * t[14 * kNtMax];
    }
    {
        vec3 r = vsub(np, c);
        I[0] += mn * (r.y * r.y + r.z * r.z); I[1] += mn * (r.x * r.x + r.z * r.z);
        I[2] += mn * (r.x * r.x + r.y * r.y); I[3] -= mn * r.x * r.y;
        I[4] -= mn * r.x * r.z; I[5] -= mn * r.y * r.z;
    }
    float reg = 1e-9f;
    float xx = I[0] + reg, yy = I[1] + reg, zz = I[2] + reg, xy = I[3], xz = I[4], yz = I[5];
    // FP64 adjugate inverse of the regularized tensor
    double X = xx, Y = yy, Z = zz, XY = xy, XZ = xz, YZ = yz;
    double a00 = Y * Z - YZ * YZ, a01 = XZ * YZ - XY * Z, a02 = XY * YZ - XZ * Y;
    double a11 = X * Z - XZ * XZ, a12 = XY * XZ - X * YZ, a22 = X * Y - XY * XY;
    double det = X * a00 + XY * a01 + XZ * a02;
    double id = 1.0 / det;
    mp->invI[0] = (float)(a00 * id); mp->invI[1] = (float)(a01 * id); mp->invI[2] = (float)(a02 * id);
    mp->invI[3] = mp->invI[1]; mp->invI[4] = (float)(a11 * id); mp->invI[5] = (float)(a12 * id);
    mp->invI[6] = mp->invI[2]; mp->invI[7] = mp->invI[5]; mp->invI[8] = (float)(a22 * id);
    mp->I[0] = xx; mp->I[1] = yy; mp->I[2] = zz; mp->I[3] = xy; mp->I[4] = xz; mp->I[5] = yz;
    mp->mass = m; mp->invmass = 1.0f / m; mp->com = c;
}

// ------------------------------------------------------------------ scenarios
// src/common.h:368-375
__device__ __forceinline__ uint32_t mix_bits(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float scen_u01(int seed, int lane) {
    return (mix_bits((uint32_t)seed * 0x9e3779b9u + (uint32_t)lane * 0x85ebca6bu) >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float scen_signed(int seed, int lane) { return scen_u01(seed, lane) * 2.0f - 1.0f; }
// (float)(seed * 37 % 97) with the 32-bit wrap of the product
__device__ __forceinline__ float seed_phase(int seed) {
    int prod = (int)((uint32_t)seed * 37u);
    return (float)(prod % 97);
}

struct Scenario { float v[kScenN]; };

// src/common.h:389-421
static __device__ __noinline__ void scenario_desc(int seed, Scenario* out) {
    float* d = out->v;
    d[S_SPEED] = 9.2f + 2.0f * scen_signed(seed, 0);
    d[S_PITCH] = 0.10f + 0.20f * scen_signed(seed, 1);
    d[S_YAW] = 0.12f * scen_signed(seed, 2);
    d[S_ROLL] = 0.16f * scen_signed(seed, 3);
    d[S_HEIGHT] = 1.75f + 0.35f * scen_signed(seed, 4);
    d[S_ROLL_RATE] = 1.8f * scen_signed(seed, 5);
    d[S_PITCH_RATE] = 1.2f * scen_signed(seed, 6);
    d[S_YAW_RATE] = 1.5f * scen_signed(seed, 7);
    d[S_AIR_RHO] = 1.225f * (0.88f + 0.22f * scen_u01(seed, 8));
    d[S_SKIN_CF] = 0.02f * (0.75f + 0.55f * scen_u01(seed, 9));
    d[S_GUST] = 0.45f + 1.10f * (0.5f + 0.5f * sinf(seed * 1.61803f));
    float phase = seed_phase(seed);
    d[S_BASE_X] = -0.25f + 1.15f * sinf(phase * 0.71f);
    d[S_BASE_Y] = 1.00f * sinf(phase * 1.13f);
    d[S_FORCE_PITCH] = 0.075f * scen_signed(seed, 10);
    d[S_FORCE_YAW] = 0.060f * scen_signed(seed, 11);
    d[S_GRIP_X] = 0.018f * scen_signed(seed, 12);
    d[S_GRIP_Y] = 0.022f * scen_signed(seed, 13);
    d[S_GRIP_Z] = 0.010f * scen_signed(seed, 14);
    d[S_MATERIAL] = 0.88f + 0.24f * scen_u01(seed, 15);
    d[S_INFILL] = 0.06f + 0.34f * scen_u01(seed, 16);
    d[S_BIAS_X] = 0.018f * scen_signed(seed, 17);
    d[S_BIAS_Y] = 0.010f * scen_signed(seed, 18);
    d[S_BIAS_Z] = 0.006f * scen_signed(seed, 19);
    d[S_SKIN_CF] *= 0.90f + 0.25f * scen_u01(seed, 20);
    d[S_WARP_PITCH] = 0.025f * scen_signed(seed, 21);
    d[S_WARP_ROLL] = 0.035f * scen_signed(seed, 22);
}

// src/common.h:423-436
__device__ __forceinline__ void point_inertia(float I[6], vec3 r, float m) {
    I[0] += m * (r.y * r.y + r.z * r.z); I[1] += m * (r.x * r.x + r.z * r.z);
    I[2] += m * (r.x * r.x + r.y * r.y); I[3] -= m * r.x * r.y;
    I[4] -= m * r.x * r.z; I[5] -= m * r.y * r.z;
}
__device__ __forceinline__ void invert_inertia(MassProps* mp) {
    float xx = mp->I[0], yy = mp->I[1], zz = mp->I[2], xy = mp->I[3], xz = mp->I[4], yz = mp->I[5];
    float det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
    float id = 1.0f / fmaxf(det, 1e-24f);
    mp->invI[0] = (yy * zz - yz * yz) * id; mp->invI[1] = (xz * yz - xy * zz) * id; mp->invI[2] = (xy * yz - xz * yy) * id;
    mp->invI[3] = mp->invI[1]; mp->invI[4] = (xx * zz - xz * xz) * id; mp->invI[5] = (xy * xz - xx * yz) * id;
    mp->invI[6] = mp->invI[2]; mp->invI[7] = mp->invI[5]; mp->invI[8] = (xx * yy - xy * xy) * id;
}
// src/common.h:441-457 (only mass and I of `src` are read)
static __device__ __noinline__ void printed_mass_props(const MassProps& src, const Scenario& sc, MassProps* out, vec3* cg_shift) {
    const float* d = sc.v;
    MassProps r = src;
    float m_shell = r.mass * d[S_MATERIAL];
    float m_fill = m_shell * d[S_INFILL];
    float m = m_shell + m_fill;
    vec3 bias = mk3(d[S_BIAS_X], d[S_BIAS_Y], d[S_BIAS_Z]);
    *cg_shift = vscl(bias, m_fill / m);
    float scale = m / r.mass;
    for (int k = 0; k < 6; k++) r.I[k] *= scale;
    point_inertia(r.I, vscl(*cg_shift, -1.0f), m_shell);
    point_inertia(r.I, vsub(bias, *cg_shift), m_fill);
    r.mass = m; r.invmass = 1.0f / m;
    r.com = vadd(r.com, *cg_shift);
    invert_inertia(&r);
    *out = r;
}

// src/common.h:459-467 with the seed-only terms (phase s, gust, base wind) passed in.
__device__ __forceinline__ vec3 wind_at(vec3 p, float t, float s, float gust, float base_x, float base_y) {
    float gx = gust * (0.55f * sinf(0.9f * p.x + 1.3f * t + s) + 0.35f * sinf(2.3f * p.z + 2.1f * t + 1.7f * s)
             + 0.25f * sinf(4.1f * p.y + 3.3f * t + 0.4f * s));
    float gy = gust * (0.50f * sinf(1.1f * p.x + 1.7f * t + 2.2f * s) + 0.30f * sinf(3.1f * p.z + 2.9f * t + 0.9f * s));
    float gz = gust * (0.30f * sinf(1.4f * p.x + 2.3f * t + 3.1f * s) + 0.20f * sinf(2.7f * p.y + 1.9f * t + 1.2f * s));
    return mk3(base_x + gx, base_y + gy, gz);
}

// ------------------------------------------------------------------ flight state
// Saved between launches for flights that outlive one; 64 B.
struct FlightState {
    vec3 pos; quat4 q; vec3 vel; vec3 wb;
    float t;       // clock (the reference restarts it at every 600-step boundary)
    int step;      // next step to integrate
    int pad;
};
static_assert(sizeof(FlightState) == 64, "FlightState is the 16-float state of the C ABI");

// Release of src/sim.cu:79-107 (launch_spread = 0).
static __device__ __noinline__ void release(const Scenario& sc, const MassProps& mp, vec3 cg_shift, FlightState* st) {
    const float* e = sc.v;
    float speed = e[S_SPEED], pitch = e[S_PITCH];
    float yaw = e[S_YAW], roll = e[S_ROLL], height = e[S_HEIGHT];
    st->pos = mk3(0, 0, height + 0);
    quat4 qyaw = qaxis(mk3(0, 0, 1), yaw);
    quat4 qpitch = qaxis(mk3(0, 1, 0), -pitch);
    quat4 qroll = qaxis(mk3(1, 0, 0), roll);
    st->q = qnormalize(qmul(qyaw, qmul(qpitch, qroll)));
    quat4 qfyaw = qaxis(mk3(0, 0, 1), yaw + e[S_FORCE_YAW]);
    quat4 qfpitch = qaxis(mk3(0, 1, 0), -(pitch + e[S_FORCE_PITCH]));
    st->vel = qrot(qmul(qfyaw, qfpitch), mk3(speed, 0, 0));
    vec3 wb = mk3(e[S_ROLL_RATE], e[S_PITCH_RATE], e[S_YAW_RATE]);
    vec3 grip = mk3(e[S_GRIP_X], e[S_GRIP_Y], e[S_GRIP_Z]);
    vec3 Jb = qrot_inv(st->q, vscl(st->vel, mp.mass));
    vec3 L = vscl(vcross(vsub(grip, cg_shift), Jb), 0.12f);
    vec3 dwr = mk3(mp.invI[0] * L.x + mp.invI[1] * L.y + mp.invI[2] * L.z,
                   mp.invI[3] * L.x + mp.invI[4] * L.y + mp.invI[5] * L.z,
                   mp.invI[6] * L.x + mp.invI[7] * L.y + mp.invI[8] * L.z);
    wb = vadd(wb, dwr);
    float w0 = vlen(wb);
    if (w0 > 35.0f) wb = vscl(wb, 35.0f / w0);
    st->wb = wb;
    st->t = 0;
    st->step = 0;
}

}  // namespace pe
