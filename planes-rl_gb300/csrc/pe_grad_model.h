// pe_grad_model.h -- the differentiable model behind pe_grad (host and device).
//
// d(objective)/d(genome) is computed in two parts:
//   * reverse mode over the flight of every (plane, scenario): a forward pass with a checkpoint
//     every K steps, then segment by segment a recompute and the hand-written adjoint of the
//     body-frame step (panel forces, integrator with its clamps, quaternion update, gusts), the
//     release and the per-flight staging (print-warped normals, CG shift) and print variation;
//     it yields the adjoint of the plane's panels (COM-relative centroid, area, unit normal),
//     mass and inertia tensor;
//   * forward mode over the plane: 35 tangent directions pushed through mesh -> mass_props ->
//     panels with dual numbers, dotted with that adjoint.
// Everything is templated on the scalar type so the same code runs on the GPU (float) and in
// host tests (double), where it is checked against central finite differences of the oracle.
//
// The differentiated distance is the landing point interpolated linearly between the last
// state above ground and the first at or below it, so it is continuous in the genome; flights
// ended by the horizon or by |y| > 300 / x < -50 use x as the reference does; oversize meshes
// (-100) and NaN flights (-10) are constant.
#pragma once
#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define PG_HD __host__ __device__ __forceinline__
#else
#define PG_HD inline
#endif

namespace pg {

// ------------------------------------------------------------------ scalar helpers
template <class T> PG_HD T p_sqrt(T x) { return sqrt(x); }
template <> PG_HD float p_sqrt<float>(float x) { return sqrtf(x); }
#ifdef __CUDA_ARCH__
// x - 2 pi round(x / 2 pi) for |x| up to a few hundred radians: Cody-Waite reduction with 2 pi
// split into its float rounding (6.2831854820251465) and the remainder (-1.7484555314695172e-7).
// The hardware sine and cosine are then within ~4e-7 absolute on [-pi, pi]; FP32 arguments near
// 100 rad already carry ~4e-6 of rounding.
__device__ __forceinline__ float reduce_2pi(float x) {
    const float k = rintf(x * 0.15915494309189535f);
    return fmaf(-k, -1.7484555314695172e-7f, fmaf(-k, 6.2831854820251465f, x));
}
#endif
template <class T> PG_HD T p_sin(T x) { return sin(x); }
template <> PG_HD float p_sin<float>(float x) {
#ifdef __CUDA_ARCH__
    return __sinf(reduce_2pi(x));
#else
    return sinf(x);
#endif
}
template <class T> PG_HD T p_cos(T x) { return cos(x); }
template <> PG_HD float p_cos<float>(float x) {
#ifdef __CUDA_ARCH__
    return __cosf(reduce_2pi(x));
#else
    return cosf(x);
#endif
}
// sqrt of a value known to be >= 0
template <class T> PG_HD T p_sqrt_nn(T x) { return sqrt(x); }
template <> PG_HD float p_sqrt_nn<float>(float x) {
#ifdef __CUDA_ARCH__
    return x > 0.f ? x * rsqrtf(x) : 0.f;
#else
    return sqrtf(x);
#endif
}
template <class T> PG_HD T p_tan(T x) { return tan(x); }
template <> PG_HD float p_tan<float>(float x) { return tanf(x); }
template <class T> PG_HD T p_rsqrt(T x) { return T(1) / sqrt(x); }
template <> PG_HD float p_rsqrt<float>(float x) {
#ifdef __CUDA_ARCH__
    return rsqrtf(x);  // <= 2 ulp
#else
    return 1.0f / sqrtf(x);
#endif
}
template <class T> PG_HD T p_rcp(T x) { return T(1) / x; }
template <> PG_HD float p_rcp<float>(float x) {
#ifdef __CUDA_ARCH__
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}
template <class T> PG_HD void p_sincos(T x, T* s, T* c) { *s = sin(x); *c = cos(x); }
template <> PG_HD void p_sincos<float>(float x, float* s, float* c) {
#ifdef __CUDA_ARCH__
    const float r = reduce_2pi(x);
    *s = __sinf(r);
    *c = __cosf(r);
#else
    *s = sinf(x);
    *c = cosf(x);
#endif
}
template <class T> PG_HD T p_abs(T x) { return x < 0 ? -x : x; }
template <class T> PG_HD T p_min(T a, T b) { return b < a ? b : a; }
template <class T> PG_HD T p_max(T a, T b) { return a < b ? b : a; }

// ------------------------------------------------------------------ dual numbers (one tangent)
template <class T>
struct Dual {
    T v, d;
    PG_HD Dual() : v(0), d(0) {}
    PG_HD Dual(T x) : v(x), d(0) {}
    PG_HD Dual(T x, T dx) : v(x), d(dx) {}
};
template <class T> PG_HD Dual<T> operator+(Dual<T> a, Dual<T> b) { return Dual<T>(a.v + b.v, a.d + b.d); }
template <class T> PG_HD Dual<T> operator-(Dual<T> a, Dual<T> b) { return Dual<T>(a.v - b.v, a.d - b.d); }
template <class T> PG_HD Dual<T> operator-(Dual<T> a) { return Dual<T>(-a.v, -a.d); }
template <class T> PG_HD Dual<T> operator*(Dual<T> a, Dual<T> b) { return Dual<T>(a.v * b.v, a.d * b.v + a.v * b.d); }
template <class T> PG_HD Dual<T> operator/(Dual<T> a, Dual<T> b) {
    T q = a.v / b.v;
    return Dual<T>(q, (a.d - q * b.d) / b.v);
}
template <class T> PG_HD Dual<T>& operator+=(Dual<T>& a, Dual<T> b) { a = a + b; return a; }
template <class T> PG_HD Dual<T>& operator-=(Dual<T>& a, Dual<T> b) { a = a - b; return a; }
template <class T> PG_HD Dual<T>& operator*=(Dual<T>& a, Dual<T> b) { a = a * b; return a; }
template <class T> PG_HD bool operator<(Dual<T> a, Dual<T> b) { return a.v < b.v; }
template <class T> PG_HD bool operator>(Dual<T> a, Dual<T> b) { return a.v > b.v; }
template <class T> PG_HD bool operator<(Dual<T> a, T b) { return a.v < b; }
template <class T> PG_HD bool operator>(Dual<T> a, T b) { return a.v > b; }
template <class T> PG_HD Dual<T> p_sqrt(Dual<T> x) {
    T s = p_sqrt(x.v);
    return Dual<T>(s, s > T(0) ? x.d / (T(2) * s) : T(0));
}
template <class T> PG_HD Dual<T> p_sin(Dual<T> x) { return Dual<T>(p_sin(x.v), p_cos(x.v) * x.d); }
template <class T> PG_HD Dual<T> p_cos(Dual<T> x) { return Dual<T>(p_cos(x.v), -p_sin(x.v) * x.d); }
template <class T> PG_HD Dual<T> p_tan(Dual<T> x) {
    T t = p_tan(x.v);
    return Dual<T>(t, (T(1) + t * t) * x.d);
}
template <class T> PG_HD Dual<T> p_abs(Dual<T> x) { return x.v < T(0) ? -x : x; }
template <class T> PG_HD Dual<T> p_min(Dual<T> a, Dual<T> b) { return b.v < a.v ? b : a; }
template <class T> PG_HD Dual<T> p_max(Dual<T> a, Dual<T> b) { return a.v < b.v ? b : a; }
template <class T> PG_HD T val(T x) { return x; }
template <class T> PG_HD T val(Dual<T> x) { return x.v; }

// ------------------------------------------------------------------ small vectors
template <class S> struct V3 { S x, y, z; };
template <class S> PG_HD V3<S> v3(S x, S y, S z) { V3<S> a; a.x = x; a.y = y; a.z = z; return a; }
template <class S> PG_HD V3<S> operator+(V3<S> a, V3<S> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class S> PG_HD V3<S> operator-(V3<S> a, V3<S> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class S> PG_HD V3<S> operator*(V3<S> a, S s) { return v3(a.x * s, a.y * s, a.z * s); }
template <class S> PG_HD S dot(V3<S> a, V3<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S> PG_HD V3<S> cross(V3<S> a, V3<S> b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ------------------------------------------------------------------ genome -> mesh (any scalar S)
// The same geometry as src/common.h:124-292; topology (decks, fin layout) is fixed by the
// genome's values and not differentiated.
enum { G_SPAN, G_CHORD, G_TAPER, G_SWEEP, G_DIH_IN, G_DIH_OUT, G_KINK, G_CAMBER1, G_CAMBER2, G_WASHOUT,
       G_ELEVATOR, G_NOSE, G_KEEL, G_DECK_GAP, G_DECK_SCALE, G_BODY, G_FIN_H, G_FIN_CHORD, G_FIN_SWEEP,
       G_TAIL_SPAN, G_TAIL_CHORD, G_TAIL_ANGLE, G_LE_B1, G_LE_B2, G_CHORD_B1, G_CHORD_B2, G_FIN_LAYOUT,
       G_FIN_CANT, G_FIN_TAPER, G_FIN_SPAN_POS, G_TAIL_SWEEP, G_TAIL_TAPER, G_TAIL_DIH, G_TIP_ROUND,
       G_CENTER_CHORD };
constexpr int kCH = 5, kSP = 8, kWingV = 102, kWingT = 160, kNtMax = 344, kNvMax = 241;

struct Topo { int nfins, fin_mode, bi, nv, nt; };
template <class S>
PG_HD Topo topology(const S* g) {
    Topo t;
    double lay = (double)val(g[G_FIN_LAYOUT]);
    t.fin_mode = lay < 0.25f ? 0 : (lay < 0.50f ? 1 : (lay < 0.75f ? 2 : 3));
    t.nfins = t.fin_mode == 2 ? 3 : (t.fin_mode == 0 ? 1 : 2);
    t.bi = val(g[G_DECK_GAP]) > 0.02f ? 1 : 0;
    t.nv = kWingV + 9 + 4 * t.nfins + 8 + (t.bi ? kWingV + 8 : 0);
    t.nt = kWingT + 8 + 2 * t.nfins + 6 + (t.bi ? kWingT + 4 : 0);
    return t;
}

template <class S>
PG_HD S camber_z(const S* g, S xc) {
    S te = g[G_ELEVATOR] * S(0.22f);
    S u = xc, v = S(1) - u;
    return S(3) * v * v * u * g[G_CAMBER1] + S(3) * v * u * u * g[G_CAMBER2] + u * u * u * te;
}
template <class S>
PG_HD void span_yz(const S* g, S t, S* y, S* z) {
    S half = g[G_SPAN] * S(0.5f);
    S b = g[G_BODY] * half, k = g[G_KINK] * half;
    if (k < b) k = b;
    S yy = S(0), zz = S(0);
    S seg = p_min(t, b);
    yy += seg;
    seg = p_min(t, k) - b;
    if (seg > S(0)) { yy += seg * p_cos(g[G_DIH_IN]); zz += seg * p_sin(g[G_DIH_IN]); }
    seg = t - k;
    if (seg > S(0)) { yy += seg * p_cos(g[G_DIH_OUT]); zz += seg * p_sin(g[G_DIH_OUT]); }
    *y = yy; *z = zz;
}
template <class S>
PG_HD V3<S> wing_pt(const S* g, S u, S xc, S zoff, S scale) {
    S half = g[G_SPAN] * S(0.5f) * scale;
    S t = p_abs(u) * half;
    S y, z;
    span_yz(g, t, &y, &z);
    S tf = p_abs(u), v = S(1) - tf;
    S cr = S(1) + g[G_CENTER_CHORD], ct = g[G_TAPER];
    S c1 = S(1) + g[G_CHORD_B1], c2 = ct + g[G_CHORD_B2];
    S ratio = v * v * v * cr + S(3) * v * v * tf * c1 + S(3) * v * tf * tf * c2 + tf * tf * tf * ct;
    S ellipse = p_sqrt(p_max(S(0.08f), S(1) - S(0.92f) * tf * tf));
    ratio *= S(1) - g[G_TIP_ROUND] + g[G_TIP_ROUND] * ellipse;
    ratio = p_max(S(0.035f), p_min(S(1.9f), ratio));
    S c = g[G_CHORD] * scale * ratio;
    S xr = S(0.5f) * g[G_CHORD] * scale * cr;
    S xt = S(0.5f) * g[G_CHORD] * scale - p_tan(g[G_SWEEP]) * half;
    S xb1 = xr + g[G_LE_B1] * g[G_CHORD] * scale;
    S xb2 = xt + g[G_LE_B2] * g[G_CHORD] * scale;
    S x_le = v * v * v * xr + S(3) * v * v * tf * xb1 + S(3) * v * tf * tf * xb2 + tf * tf * tf * xt;
    S x = x_le - xc * c;
    S zc = z * scale + camber_z(g, xc) * c;
    S x_c4 = x_le - S(0.25f) * c;
    zc += g[G_WASHOUT] * tf * (x - x_c4);
    return v3(x, val(u) < 0 ? -y : y, zc + zoff);
}

template <class S>
PG_HD V3<S> mesh_vertex(const S* g, const Topo& tp, int idx) {
    if (idx < kWingV) {
        int i = idx / (kCH + 1), j = idx % (kCH + 1);
        return wing_pt(g, S((double)(i - kSP) / kSP), S((double)j / kCH), S(0), S(1));
    }
    idx -= kWingV;
    S hs = S(0.5f) * g[G_SPAN] * g[G_TAIL_SPAN];
    S z0 = camber_z(g, S(0.82f)) * g[G_CHORD];
    if (idx < 9) {
        int i = idx / 3, j = idx % 3;
        S hc = g[G_CHORD] * g[G_TAIL_CHORD];
        S x0 = S(-0.32f) * g[G_CHORD];
        S u = S((double)(i - 1)), au = p_abs(u);
        S tc = hc * (S(1) + (g[G_TAIL_TAPER] - S(1)) * au);
        S xle = x0 - g[G_TAIL_SWEEP] * hc * au;
        S x = xle - S(0.5 * j) * tc;
        S z = z0 + g[G_TAIL_ANGLE] * (x - xle) + au * hs * p_sin(g[G_TAIL_DIH]);
        return v3(x, u * hs * p_cos(g[G_TAIL_DIH]), z);
    }
    idx -= 9;
    if (idx < 4 * tp.nfins) {
        int f = idx >> 2, c = idx & 3;
        S y0, zb;
        int side;
        if (tp.fin_mode == 3) {
            S yo = hs * S(0.94f) * p_cos(g[G_TAIL_DIH]);
            S zo = z0 + hs * S(0.94f) * p_sin(g[G_TAIL_DIH]);
            side = f == 0 ? -1 : 1; y0 = f == 0 ? -yo : yo; zb = zo;
        } else {
            int k = tp.fin_mode == 1 ? f + 1 : f;
            if (k == 0) { side = 0; y0 = S(0); zb = z0; }
            else {
                S yp = hs * g[G_FIN_SPAN_POS] * p_cos(g[G_TAIL_DIH]);
                S zp = z0 + hs * g[G_FIN_SPAN_POS] * p_sin(g[G_TAIL_DIH]);
                side = k == 1 ? -1 : 1; y0 = k == 1 ? -yp : yp; zb = zp;
            }
        }
        S fc = g[G_CHORD] * g[G_FIN_CHORD];
        S xr = S(-0.32f) * g[G_CHORD] - g[G_TAIL_CHORD] * g[G_CHORD] * S(0.82f);
        if (c < 2) return v3(c == 0 ? xr + S(0.5f) * fc : xr - S(0.5f) * fc, y0, zb);
        S sweep = fc * g[G_FIN_SWEEP], tipc = fc * g[G_FIN_TAPER];
        S cant = side == 0 ? S(0) : g[G_FIN_CANT];
        S ya = y0 + S((double)side) * p_sin(cant) * g[G_FIN_H];
        S za = zb + p_cos(cant) * g[G_FIN_H];
        return v3(c == 2 ? xr - sweep + S(0.5f) * tipc : xr - sweep - S(0.5f) * tipc, ya, za);
    }
    idx -= 4 * tp.nfins;
    if (tp.bi) {
        if (idx < kWingV) {
            int i = idx / (kCH + 1), j = idx % (kCH + 1);
            return wing_pt(g, S((double)(i - kSP) / kSP), S((double)j / kCH), g[G_DECK_GAP], g[G_DECK_SCALE]);
        }
        idx -= kWingV;
    }
    if (idx < 8) {
        int j = idx >> 1;
        S xc = S((double)j / 3);
        V3<S> top = wing_pt(g, S(0), xc, S(0), S(1));
        if ((idx & 1) == 0) return top;
        return v3(top.x, S(0), top.z - g[G_KEEL] * (S(0.35f) + S(0.65f) * xc));
    }
    idx -= 8;
    S sgn = S((idx >> 2) == 0 ? -1.0 : 1.0);
    int c = idx & 3;
    S u = sgn * g[G_KINK];
    if (c == 0) return wing_pt(g, u, S(0.25f), S(0), S(1));
    if (c == 1) return wing_pt(g, u, S(0.55f), S(0), S(1));
    return wing_pt(g, u, c == 2 ? S(0.25f) : S(0.55f), g[G_DECK_GAP], g[G_DECK_SCALE]);
}

PG_HD void mesh_tri(const Topo& tp, int t, int* ia, int* ib, int* ic) {
    int vb = 0;
    if (t < kWingT) goto grid;
    t -= kWingT; vb = kWingV;
    if (t < 8) {
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
    if (t < 6) {
        int a = vb + (t >> 1) * 2;
        if (t & 1) { *ia = a + 1; *ib = a + 3; *ic = a + 2; } else { *ia = a; *ib = a + 1; *ic = a + 2; }
        return;
    }
    t -= 6; vb += 8;
    {
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

// Mass properties, src/common.h:311-365, as per-triangle terms and the steps between the two
// passes (so they can be summed serially or by a thread block).
// Pass 1, triangle i: shell mass mi and its first moment (a + b + d) mi / 3.
template <class S>
PG_HD void tri_mass(const V3<S>* V, const Topo& tp, int i, S* mi, V3<S>* mc) {
    int ia, ib, ic;
    mesh_tri(tp, i, &ia, &ib, &ic);
    V3<S> a = V[ia], b = V[ib], d = V[ic];
    V3<S> n = cross(b - a, d - a);
    *mi = S(0.5f) * p_sqrt(dot(n, n)) * S(1240.0f * 0.00045f);
    *mc = (a + b + d) * (*mi * S(1.0 / 3));
}
// Between the passes: add the nose mass and divide by the total (shell mass m, moment c in; total
// mass, COM and the nose point mass out).
template <class S>
PG_HD void mass_com(const S* g, S* m, V3<S>* c, S* mn, V3<S>* np) {
    *np = v3(S(0.5f) * g[G_CHORD], S(0), S(0));
    *mn = g[G_NOSE] * *m;
    *m = *m + *mn;
    *c = (*c + *np * *mn) * (S(1) / *m);
}
// Pass 2, triangle i: its inertia about the COM c (thin-shell membrane + wall thickness), added to I.
template <class S>
PG_HD void tri_inertia(const V3<S>* V, const Topo& tp, int i, V3<S> c, S I[6]) {
    const S rho = S(1240.0f * 0.00045f);
    const S w2 = S(0.00045f * 0.00045f / 12.0);
    int ia, ib, ic;
    mesh_tri(tp, i, &ia, &ib, &ic);
    V3<S> a = V[ia] - c, b = V[ib] - c, d = V[ic] - c;
    V3<S> n = cross(b - a, d - a);
    S nl = p_sqrt(dot(n, n));
    S mi = S(0.5f) * nl * rho;
    S exx = (a.x * a.x + b.x * b.x + d.x * d.x + a.x * b.x + a.x * d.x + b.x * d.x) * S(1.0 / 6);
    S eyy = (a.y * a.y + b.y * b.y + d.y * d.y + a.y * b.y + a.y * d.y + b.y * d.y) * S(1.0 / 6);
    S ezz = (a.z * a.z + b.z * b.z + d.z * d.z + a.z * b.z + a.z * d.z + b.z * d.z) * S(1.0 / 6);
    S exy = (S(2) * (a.x * a.y + b.x * b.y + d.x * d.y) + a.x * b.y + b.x * a.y + a.x * d.y + d.x * a.y +
             b.x * d.y + d.x * b.y) * S(1.0 / 12);
    S exz = (S(2) * (a.x * a.z + b.x * b.z + d.x * d.z) + a.x * b.z + b.x * a.z + a.x * d.z + d.x * a.z +
             b.x * d.z + d.x * b.z) * S(1.0 / 12);
    S eyz = (S(2) * (a.y * a.z + b.y * b.z + d.y * d.z) + a.y * b.z + b.y * a.z + a.y * d.z + d.y * a.z +
             b.y * d.z + d.y * b.z) * S(1.0 / 12);
    I[0] += mi * (eyy + ezz); I[1] += mi * (exx + ezz); I[2] += mi * (exx + eyy);
    I[3] -= mi * exy; I[4] -= mi * exz; I[5] -= mi * eyz;
    S th = mi * w2;
    if (val(nl) > 1e-12) {
        V3<S> nn = n * (S(1) / nl);
        I[0] += th * (S(1) - nn.x * nn.x); I[1] += th * (S(1) - nn.y * nn.y); I[2] += th * (S(1) - nn.z * nn.z);
        I[3] -= th * nn.x * nn.y; I[4] -= th * nn.x * nn.z; I[5] -= th * nn.y * nn.z;
    } else {  // the reference's norm3 falls back to (0, 0, 1)
        I[0] += th; I[1] += th;
    }
}
// After pass 2: the nose point mass and the 1e-9 regularization of the diagonal.
template <class S>
PG_HD void inertia_finish(S mn, V3<S> np, V3<S> c, S I[6]) {
    V3<S> r = np - c;
    I[0] += mn * (r.y * r.y + r.z * r.z); I[1] += mn * (r.x * r.x + r.z * r.z);
    I[2] += mn * (r.x * r.x + r.y * r.y); I[3] -= mn * r.x * r.y;
    I[4] -= mn * r.x * r.z; I[5] -= mn * r.y * r.z;
    I[0] += S(1e-9f); I[1] += S(1e-9f); I[2] += S(1e-9f);
}

// Mass, COM and inertia about the COM (xx yy zz xy xz yz, regularized), serially.
template <class S>
PG_HD void mass_props(const S* g, const V3<S>* V, const Topo& tp, S* mass, V3<S>* com, S I[6]) {
    S m = S(0);
    V3<S> c = v3(S(0), S(0), S(0));
    for (int i = 0; i < tp.nt; i++) {
        S mi;
        V3<S> mc;
        tri_mass(V, tp, i, &mi, &mc);
        m += mi;
        c = c + mc;
    }
    S mn;
    V3<S> np;
    mass_com(g, &m, &c, &mn, &np);
    for (int k = 0; k < 6; k++) I[k] = S(0);
    for (int i = 0; i < tp.nt; i++) tri_inertia(V, tp, i, c, I);
    inertia_finish(mn, np, c, I);
    *mass = m;
    *com = c;
}

// COM-relative centroid, area and unit normal of triangle t (src/sim.cu:40-48).
template <class S>
PG_HD void panel(const V3<S>* V, const Topo& tp, V3<S> com, int t, V3<S>* ct, S* A, V3<S>* n) {
    int ia, ib, ic;
    mesh_tri(tp, t, &ia, &ib, &ic);
    V3<S> a = V[ia] - com, b = V[ib] - com, d = V[ic] - com;
    V3<S> nrm = cross(b - a, d - a);
    S nl = p_sqrt(dot(nrm, nrm));
    *A = S(0.5f) * nl;
    *ct = (a + b + d) * S(1.0 / 3);
    *n = val(nl) > 2e-12 ? nrm * (S(1) / nl) : v3(S(0), S(0), S(1));
}


// ------------------------------------------------------------------ flight (scalar T)
constexpr float kDt = 1.0f / 600.0f;
constexpr float kGrav = 9.81f;

template <class T> struct M3 { T a[3][3]; };

// Constants of one flight after print variation (src/common.h:441-457) and the scenario draw.
template <class T>
struct FlightP {
    T mass, invmass, I[6], invI[9];
    T cf, gust, phase, base_x, base_y;
};

template <class T>
struct St { V3<T> pos; T q[4]; V3<T> vel, w; T t; };

template <class T>
PG_HD void rot_rows(const T q[4], M3<T>& R) {
    T w = q[0], x = q[1], y = q[2], z = q[3];
    R.a[0][0] = T(1) - T(2) * (y * y + z * z); R.a[0][1] = T(2) * (x * y - w * z); R.a[0][2] = T(2) * (x * z + w * y);
    R.a[1][0] = T(2) * (x * y + w * z); R.a[1][1] = T(1) - T(2) * (x * x + z * z); R.a[1][2] = T(2) * (y * z - w * x);
    R.a[2][0] = T(2) * (x * z - w * y); R.a[2][1] = T(2) * (y * z + w * x); R.a[2][2] = T(1) - T(2) * (x * x + y * y);
}

// Gusts (src/common.h:459-467) and, optionally, their Jacobian wrt position (J[i][j] = dW_i/dp_j).
template <class T>
PG_HD V3<T> wind(const FlightP<T>& P, V3<T> p, T t, T J[3][3]) {
    const T s = P.phase, G = P.gust;
    T a1 = T(0.9f) * p.x + T(1.3f) * t + s, a2 = T(2.3f) * p.z + T(2.1f) * t + T(1.7f) * s;
    T a3 = T(4.1f) * p.y + T(3.3f) * t + T(0.4f) * s, b1 = T(1.1f) * p.x + T(1.7f) * t + T(2.2f) * s;
    T b2 = T(3.1f) * p.z + T(2.9f) * t + T(0.9f) * s, c1 = T(1.4f) * p.x + T(2.3f) * t + T(3.1f) * s;
    T c2 = T(2.7f) * p.y + T(1.9f) * t + T(1.2f) * s;
    T sa1, sa2, sa3, sb1, sb2, sc1, sc2;
    if (J) {
        T ca1, ca2, ca3, cb1, cb2, cc1, cc2;
        p_sincos(a1, &sa1, &ca1); p_sincos(a2, &sa2, &ca2); p_sincos(a3, &sa3, &ca3);
        p_sincos(b1, &sb1, &cb1); p_sincos(b2, &sb2, &cb2); p_sincos(c1, &sc1, &cc1); p_sincos(c2, &sc2, &cc2);
        J[0][0] = G * T(0.55f * 0.9f) * ca1; J[0][1] = G * T(0.25f * 4.1f) * ca3; J[0][2] = G * T(0.35f * 2.3f) * ca2;
        J[1][0] = G * T(0.50f * 1.1f) * cb1; J[1][1] = T(0); J[1][2] = G * T(0.30f * 3.1f) * cb2;
        J[2][0] = G * T(0.30f * 1.4f) * cc1; J[2][1] = G * T(0.20f * 2.7f) * cc2; J[2][2] = T(0);
    } else {
        sa1 = p_sin(a1); sa2 = p_sin(a2); sa3 = p_sin(a3); sb1 = p_sin(b1); sb2 = p_sin(b2);
        sc1 = p_sin(c1); sc2 = p_sin(c2);
    }
    T gx = G * (T(0.55f) * sa1 + T(0.35f) * sa2 + T(0.25f) * sa3);
    T gy = G * (T(0.50f) * sb1 + T(0.30f) * sb2);
    T gz = G * (T(0.30f) * sc1 + T(0.20f) * sc2);
    return v3(P.base_x + gx, P.base_y + gy, gz);
}

// Per-step quantities shared by every panel.
template <class T>
struct Pre { M3<T> R; V3<T> va, vb, w; };

// J (optional) receives the gust Jacobian at the state's position for step_pre_adj.
template <class T>
PG_HD void step_pre(const FlightP<T>& P, const St<T>& s, Pre<T>& pr, T (*J)[3] = nullptr) {
    rot_rows(s.q, pr.R);
    V3<T> wd = wind(P, s.pos, s.t, J);
    pr.va = s.vel - wd;
    for (int j = 0; j < 3; j++)  // vb = R^T va
        (&pr.vb.x)[j] = pr.R.a[0][j] * pr.va.x + pr.R.a[1][j] * pr.va.y + pr.R.a[2][j] * pr.va.z;
    pr.w = s.w;
}

// Force f and torque rb x f of one panel in the body frame.
template <class T>
PG_HD void panel_fwd(const Pre<T>& pr, V3<T> rb, V3<T> nb, T ak, T cf, V3<T>* f, V3<T>* tq) {
    V3<T> vr = pr.vb + cross(pr.w, rb);
    T V2 = dot(vr, vr);
    if (V2 < T(1e-6f)) { *f = v3(T(0), T(0), T(0)); *tq = *f; return; }
    T inv = p_rsqrt(V2);
    T s = dot(vr, nb) * inv;
    T qd = V2 * ak;
    T sq = p_sqrt_nn(p_max(T(0), T(1) - s * s));
    T na = qd * s * (T(1.9f) * sq + T(2) * p_abs(s) - cf);
    T nv = qd * cf * inv;
    *f = v3(-(na * nb.x + nv * vr.x), -(na * nb.y + nv * vr.y), -(na * nb.z + nv * vr.z));
    *tq = cross(rb, *f);
}

// Adjoint of panel_fwd for the step's force / torque adjoints LF, LT.  Accumulates the panel's
// adjoints (Lrb, Lnb, Lak) and this panel's share of the step's Lvb, Lw.
template <class T>
PG_HD void panel_adj(const Pre<T>& pr, V3<T> rb, V3<T> nb, T ak, T cf, V3<T> LF, V3<T> LT, V3<T>* Lrb, V3<T>* Lnb,
                     T* Lak, V3<T>* Lvb, V3<T>* Lw) {
    V3<T> vr = pr.vb + cross(pr.w, rb);
    T V2 = dot(vr, vr);
    if (V2 < T(1e-6f)) return;
    T inv = p_rsqrt(V2);
    T vn = dot(vr, nb);
    T s = vn * inv;
    T qd = V2 * ak;
    T u = T(1) - s * s;
    T sq = p_sqrt_nn(p_max(T(0), u));
    T as = p_abs(s);
    T gf = T(1.9f) * sq + T(2) * as - cf;
    T na = qd * s * gf;
    T nv = qd * cf * inv;
    V3<T> f = v3(-(na * nb.x + nv * vr.x), -(na * nb.y + nv * vr.y), -(na * nb.z + nv * vr.z));
    // T += rb x f ; F += f
    V3<T> Lf = LF + cross(LT, rb);
    *Lrb = *Lrb + cross(f, LT);
    V3<T> Lnf = v3(-Lf.x, -Lf.y, -Lf.z);
    T Lna = dot(Lnf, nb);
    *Lnb = *Lnb + Lnf * na;
    T Lnv = dot(Lnf, vr);
    V3<T> Lvr = Lnf * nv;
    T Lqd = Lnv * cf * inv + Lna * s * gf;
    T Linv = Lnv * qd * cf;
    T Ls = Lna * qd * gf;
    T Lgf = Lna * qd * s;
    T Lsq = T(1.9f) * Lgf;
    Ls += T(2) * (s < T(0) ? T(-1) : T(1)) * Lgf;
    if (u > T(0) && sq > T(1e-6f)) Ls -= Lsq * s * p_rcp(sq);
    T LV2 = Lqd * ak;
    *Lak += Lqd * V2;
    T Lvn = Ls * inv;
    Linv += Ls * vn;
    Lvr = Lvr + nb * Lvn;
    *Lnb = *Lnb + vr * Lvn;
    LV2 += Linv * (T(-0.5f) * inv * inv * inv);
    Lvr = Lvr + vr * (T(2) * LV2);
    *Lvb = *Lvb + Lvr;
    *Lw = *Lw + cross(rb, Lvr);
    *Lrb = *Lrb + cross(Lvr, pr.w);
}

// x scaled down to length L when longer (compared as squared lengths).
template <class T>
PG_HD V3<T> clamp_len(V3<T> x, T L) {
    T l2 = dot(x, x);
    return l2 > L * L ? x * (L * p_rsqrt(l2)) : x;
}
template <class T>
PG_HD V3<T> clamp_len_adj(V3<T> x, T L, V3<T> lam) {
    T l2 = dot(x, x);
    if (!(l2 > L * L)) return lam;
    T il = p_rsqrt(l2);
    return (lam - x * (dot(x, lam) * il * il)) * (L * il);
}

// The intermediates of one integrator step that its adjoint reads.
template <class T>
struct PostF {
    V3<T> Fw, Iw, tq, w1, wn, vel1;  // world force with gravity, I w, net torque, w before / after its clamp, v before its clamp
    T qo[4], il;                     // the normalized attitude and 1 / |q + h dq|
};

// The integrator, src/sim.cu:177-197 (body torque, world force), from the attitude matrix R of
// s; returns the next state and keeps its intermediates in f.
template <class T>
PG_HD St<T> step_post_f(const FlightP<T>& P, const St<T>& s, const M3<T>& R, V3<T> Fb, V3<T> Tb, PostF<T>& f) {
    const T dt = T(kDt);
    V3<T> Fw;
    for (int i = 0; i < 3; i++) (&Fw.x)[i] = R.a[i][0] * Fb.x + R.a[i][1] * Fb.y + R.a[i][2] * Fb.z;
    Fw.z = Fw.z - P.mass * T(kGrav);
    V3<T> w = s.w;
    V3<T> Iw = v3(P.I[0] * w.x + P.I[3] * w.y + P.I[4] * w.z, P.I[3] * w.x + P.I[1] * w.y + P.I[5] * w.z,
                  P.I[4] * w.x + P.I[5] * w.y + P.I[2] * w.z);
    V3<T> tq = Tb - cross(w, Iw);
    V3<T> dw = v3(P.invI[0] * tq.x + P.invI[1] * tq.y + P.invI[2] * tq.z,
                  P.invI[3] * tq.x + P.invI[4] * tq.y + P.invI[5] * tq.z,
                  P.invI[6] * tq.x + P.invI[7] * tq.y + P.invI[8] * tq.z);
    St<T> n;
    const V3<T> w1 = w + dw * dt;
    n.w = clamp_len(w1, T(150));
    const V3<T> vel1 = s.vel + Fw * (P.invmass * dt);
    n.vel = clamp_len(vel1, T(60));
    n.pos = s.pos + n.vel * dt;
    const T* q = s.q;
    T dq[4] = {-(q[1] * n.w.x + q[2] * n.w.y + q[3] * n.w.z), q[0] * n.w.x + q[2] * n.w.z - q[3] * n.w.y,
               q[0] * n.w.y - q[1] * n.w.z + q[3] * n.w.x, q[0] * n.w.z + q[1] * n.w.y - q[2] * n.w.x};
    T h = T(0.5f) * dt, qn[4], l2 = T(0);
    for (int k = 0; k < 4; k++) { qn[k] = q[k] + h * dq[k]; l2 += qn[k] * qn[k]; }
    T il = p_rsqrt(l2);
    for (int k = 0; k < 4; k++) n.q[k] = qn[k] * il;
    n.t = s.t + dt;
    f.Fw = Fw; f.Iw = Iw; f.tq = tq; f.w1 = w1; f.wn = n.w; f.vel1 = vel1;
    for (int k = 0; k < 4; k++) f.qo[k] = n.q[k];
    f.il = il;
    return n;
}

// The integrator; returns the next state.
template <class T>
PG_HD St<T> step_post(const FlightP<T>& P, const St<T>& s, const Pre<T>& pr, V3<T> Fb, V3<T> Tb) {
    PostF<T> f;
    return step_post_f(P, s, pr.R, Fb, Tb, f);
}

// Parameter adjoints of one flight.
template <class T>
struct LamP { T mass, invmass, I[6], invI[9]; };

// Adjoint of the integrator from its intermediates f (step_post_f of the same s, R, Fb, Tb): from
// the next state's adjoint L1 to the adjoint of s (accumulated into L0, which the caller zeroes or
// seeds) and of Fb, Tb, R and the parameters.
template <class T>
PG_HD void step_post_adj_f(const FlightP<T>& P, const St<T>& s, const M3<T>& R, V3<T> Fb, const PostF<T>& f,
                           const St<T>& L1, St<T>& L0, V3<T>* LFb, V3<T>* LTb, M3<T>& LR, LamP<T>& LP) {
    const T dt = T(kDt);
    const V3<T> w = s.w, wn = f.wn, Iw = f.Iw;
    const T* q = s.q;
    const T* qo = f.qo;
    const T il = f.il, h = T(0.5f) * dt;
    // q' = qn / |qn|
    T qdot = L1.q[0] * qo[0] + L1.q[1] * qo[1] + L1.q[2] * qo[2] + L1.q[3] * qo[3];
    T Lqn[4];
    for (int k = 0; k < 4; k++) Lqn[k] = (L1.q[k] - qo[k] * qdot) * il;
    // qn = q + h M(w') q  and = q + h N(q) w'
    T Lq[4] = {Lqn[0], Lqn[1], Lqn[2], Lqn[3]};
    // M^T Lqn, M rows (w x y z) x cols (qw qx qy qz)
    Lq[0] += h * (wn.x * Lqn[1] + wn.y * Lqn[2] + wn.z * Lqn[3]);
    Lq[1] += h * (-wn.x * Lqn[0] - wn.z * Lqn[2] + wn.y * Lqn[3]);
    Lq[2] += h * (-wn.y * Lqn[0] + wn.z * Lqn[1] - wn.x * Lqn[3]);
    Lq[3] += h * (-wn.z * Lqn[0] - wn.y * Lqn[1] + wn.x * Lqn[2]);
    V3<T> Lwn = L1.w;
    Lwn.x += h * (-q[1] * Lqn[0] + q[0] * Lqn[1] + q[3] * Lqn[2] - q[2] * Lqn[3]);
    Lwn.y += h * (-q[2] * Lqn[0] - q[3] * Lqn[1] + q[0] * Lqn[2] + q[1] * Lqn[3]);
    Lwn.z += h * (-q[3] * Lqn[0] + q[2] * Lqn[1] - q[1] * Lqn[2] + q[0] * Lqn[3]);
    // pos' = pos + dt vel'
    L0.pos = L0.pos + L1.pos;
    V3<T> Lveln = L1.vel + L1.pos * dt;
    V3<T> Lvel1 = clamp_len_adj(f.vel1, T(60), Lveln);
    L0.vel = L0.vel + Lvel1;
    V3<T> LFw = Lvel1 * (P.invmass * dt);
    LP.invmass += dt * dot(Lvel1, f.Fw);
    LP.mass += -T(kGrav) * LFw.z;
    V3<T> Lw1 = clamp_len_adj(f.w1, T(150), Lwn);
    V3<T> Lw = Lw1;
    V3<T> Ldw = Lw1 * dt;
    V3<T> Ltq = v3(P.invI[0] * Ldw.x + P.invI[3] * Ldw.y + P.invI[6] * Ldw.z,
                   P.invI[1] * Ldw.x + P.invI[4] * Ldw.y + P.invI[7] * Ldw.z,
                   P.invI[2] * Ldw.x + P.invI[5] * Ldw.y + P.invI[8] * Ldw.z);
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) LP.invI[r * 3 + c] += (&Ldw.x)[r] * (&f.tq.x)[c];
    *LTb = Ltq;
    V3<T> Lgy = v3(-Ltq.x, -Ltq.y, -Ltq.z);
    // gyro = w x Iw
    Lw = Lw + cross(Iw, Lgy);
    V3<T> LIw = cross(Lgy, w);
    Lw = Lw + v3(P.I[0] * LIw.x + P.I[3] * LIw.y + P.I[4] * LIw.z, P.I[3] * LIw.x + P.I[1] * LIw.y + P.I[5] * LIw.z,
                 P.I[4] * LIw.x + P.I[5] * LIw.y + P.I[2] * LIw.z);
    LP.I[0] += LIw.x * w.x; LP.I[1] += LIw.y * w.y; LP.I[2] += LIw.z * w.z;
    LP.I[3] += LIw.x * w.y + LIw.y * w.x; LP.I[4] += LIw.x * w.z + LIw.z * w.x; LP.I[5] += LIw.y * w.z + LIw.z * w.y;
    L0.w = L0.w + Lw;
    // Fw0 = R Fb
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) LR.a[i][j] += (&LFw.x)[i] * (&Fb.x)[j];
    for (int j = 0; j < 3; j++)
        (&LFb->x)[j] = R.a[0][j] * LFw.x + R.a[1][j] * LFw.y + R.a[2][j] * LFw.z;
    for (int k = 0; k < 4; k++) L0.q[k] += Lq[k];
}

// Adjoint of step_post: its intermediates recomputed, then step_post_adj_f.
template <class T>
PG_HD void step_post_adj(const FlightP<T>& P, const St<T>& s, const Pre<T>& pr, V3<T> Fb, V3<T> Tb, const St<T>& L1,
                         St<T>& L0, V3<T>* LFb, V3<T>* LTb, M3<T>& LR, LamP<T>& LP) {
    PostF<T> f;
    (void)step_post_f(P, s, pr.R, Fb, Tb, f);
    step_post_adj_f(P, s, pr.R, Fb, f, L1, L0, LFb, LTb, LR, LP);
}

// Adjoint of step_pre given the step's summed panel adjoints Lvb, Lw_panels and LR from
// step_post_adj.
template <class T>
PG_HD void step_pre_adj(const FlightP<T>& P, const St<T>& s, const Pre<T>& pr, V3<T> Lvb, V3<T> Lwp, M3<T>& LR,
                        St<T>& L0, const T (*Jin)[3] = nullptr) {
    // vb = R^T va
    V3<T> Lva;
    for (int i = 0; i < 3; i++) (&Lva.x)[i] = pr.R.a[i][0] * Lvb.x + pr.R.a[i][1] * Lvb.y + pr.R.a[i][2] * Lvb.z;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) LR.a[i][j] += (&pr.va.x)[i] * (&Lvb.x)[j];
    L0.vel = L0.vel + Lva;
    T J[3][3];
    if (Jin) {
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) J[i][j] = Jin[i][j];
    } else {
        wind(P, s.pos, s.t, J);
    }
    // va = vel - W(pos)  ->  Lpos -= J^T Lva
    L0.pos.x -= J[0][0] * Lva.x + J[1][0] * Lva.y + J[2][0] * Lva.z;
    L0.pos.y -= J[0][1] * Lva.x + J[1][1] * Lva.y + J[2][1] * Lva.z;
    L0.pos.z -= J[0][2] * Lva.x + J[1][2] * Lva.y + J[2][2] * Lva.z;
    L0.w = L0.w + Lwp;
    // R(q)
    const T w = s.q[0], x = s.q[1], y = s.q[2], z = s.q[3];
    const T (*G)[3] = LR.a;
    L0.q[0] += T(2) * (-z * G[0][1] + y * G[0][2] + z * G[1][0] - x * G[1][2] - y * G[2][0] + x * G[2][1]);
    L0.q[1] += T(2) * (y * G[0][1] + z * G[0][2] + y * G[1][0] - T(2) * x * G[1][1] - w * G[1][2] + z * G[2][0] +
                       w * G[2][1] - T(2) * x * G[2][2]);
    L0.q[2] += T(2) * (-T(2) * y * G[0][0] + x * G[0][1] + w * G[0][2] + x * G[1][0] + z * G[1][2] - w * G[2][0] +
                       z * G[2][1] - T(2) * y * G[2][2]);
    L0.q[3] += T(2) * (-T(2) * z * G[0][0] - w * G[0][1] + x * G[0][2] + w * G[1][0] - T(2) * z * G[1][1] +
                       y * G[1][2] + x * G[2][0] + y * G[2][1]);
}

// Landing: the reference's termination (src/sim.cu:198-204) and the interpolated distance.
// Returns 1 when the flight ends at this step; *kind: 1 ground, 2 other bound or horizon, 3 NaN.
template <class T>
PG_HD int terminate(const St<T>& before, const St<T>& after, int step, int max_steps, T* d, int* kind) {
    const V3<T> p = after.pos, v = after.vel;
    bool bad = !(p.x == p.x && v.x == v.x);
    if (bad) { *d = T(-10); *kind = 3; return 1; }
    if (p.z <= T(0)) {
        T z0 = before.pos.z, z1 = p.z;
        T a = z0 / (z0 - z1);
        *d = before.pos.x + (p.x - before.pos.x) * a;
        *kind = 1;
        return 1;
    }
    if (p_abs(p.y) > T(300) || p.x < T(-50) || step == max_steps - 1) { *d = p.x; *kind = 2; return 1; }
    return 0;
}
// Adjoint seeds of the distance wrt the last two states.
template <class T>
PG_HD void terminate_adj(const St<T>& before, const St<T>& after, int kind, St<T>& Lbefore, St<T>& Lafter) {
    if (kind == 1) {
        T x0 = before.pos.x, z0 = before.pos.z, x1 = after.pos.x, z1 = after.pos.z;
        T den = z0 - z1, a = z0 / den;
        Lafter.pos.x += a;
        Lbefore.pos.x += T(1) - a;
        Lbefore.pos.z += (x1 - x0) * (-z1) / (den * den);
        Lafter.pos.z += (x1 - x0) * z0 / (den * den);
    } else if (kind == 2) {
        Lafter.pos.x += T(1);
    }
}

// ------------------------------------------------------------------ per-flight set-up and its adjoint
// Scenario fields used here (src/common.h:377-387 order).
enum { SC_SPEED, SC_PITCH, SC_YAW, SC_ROLL, SC_HEIGHT, SC_RR, SC_PR, SC_YR, SC_RHO, SC_CF, SC_GUST, SC_BX, SC_BY,
       SC_FP, SC_FY, SC_GX, SC_GY, SC_GZ, SC_MAT, SC_INF, SC_BIASX, SC_BIASY, SC_BIASZ, SC_WP, SC_WR };

// Print variation of (mass, I) and its linear coefficients: I' = sigma I + mass beta.
template <class T>
PG_HD void printed(const T* sc, T mass, const T I[6], FlightP<T>& P, V3<T>* cg, T* sigma, T beta[6]) {
    T ms = sc[SC_MAT], inf = sc[SC_INF];
    T m_shell = mass * ms, m_fill = m_shell * inf, m = m_shell + m_fill;
    V3<T> bias = v3(sc[SC_BIASX], sc[SC_BIASY], sc[SC_BIASZ]);
    *cg = bias * (inf / (T(1) + inf));
    *sigma = ms * (T(1) + inf);
    V3<T> r1 = v3(-cg->x, -cg->y, -cg->z), r2 = bias - *cg;
    T P1[6] = {r1.y * r1.y + r1.z * r1.z, r1.x * r1.x + r1.z * r1.z, r1.x * r1.x + r1.y * r1.y, -r1.x * r1.y,
               -r1.x * r1.z, -r1.y * r1.z};
    T P2[6] = {r2.y * r2.y + r2.z * r2.z, r2.x * r2.x + r2.z * r2.z, r2.x * r2.x + r2.y * r2.y, -r2.x * r2.y,
               -r2.x * r2.z, -r2.y * r2.z};
    for (int k = 0; k < 6; k++) {
        beta[k] = ms * P1[k] + ms * inf * P2[k];
        P.I[k] = *sigma * I[k] + mass * beta[k];
    }
    P.mass = m;
    P.invmass = T(1) / m;
    // inverse of the symmetric tensor (adjugate), in FP64 whatever T is
    double xx = P.I[0], yy = P.I[1], zz = P.I[2], xy = P.I[3], xz = P.I[4], yz = P.I[5];
    double det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
    double id = 1.0 / det;
    P.invI[0] = T((yy * zz - yz * yz) * id); P.invI[1] = T((xz * yz - xy * zz) * id);
    P.invI[2] = T((xy * yz - xz * yy) * id); P.invI[3] = P.invI[1]; P.invI[4] = T((xx * zz - xz * xz) * id);
    P.invI[5] = T((xy * xz - xx * yz) * id); P.invI[6] = P.invI[2]; P.invI[7] = P.invI[5];
    P.invI[8] = T((xx * yy - xy * xy) * id);
    P.cf = sc[SC_CF];
    P.gust = sc[SC_GUST];
    P.base_x = sc[SC_BX];
    P.base_y = sc[SC_BY];
}

// Adjoint of printed(): from LP (adjoints of mass', invmass', I', invI') to (mass, I).  The
// inverse's adjoint, -inv^T G inv^T, is formed in double.
template <class T>
PG_HD void printed_adj(const FlightP<T>& P, T sigma, const T beta[6], const LamP<T>& LP, T* Lmass, T LI[6]) {
    double inv[3][3], G[3][3], H[3][3], out[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) { inv[r][c] = (double)P.invI[r * 3 + c]; G[r][c] = (double)LP.invI[r * 3 + c]; }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            double a = 0;
            for (int k = 0; k < 3; k++) a += G[r][k] * inv[k][c];
            H[r][c] = a;
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            double a = 0;
            for (int k = 0; k < 3; k++) a += inv[r][k] * H[k][c];
            out[r][c] = -a;
        }
    T LIp[6];
    LIp[0] = LP.I[0] + (T)out[0][0]; LIp[1] = LP.I[1] + (T)out[1][1]; LIp[2] = LP.I[2] + (T)out[2][2];
    LIp[3] = LP.I[3] + (T)(out[0][1] + out[1][0]); LIp[4] = LP.I[4] + (T)(out[0][2] + out[2][0]);
    LIp[5] = LP.I[5] + (T)(out[1][2] + out[2][1]);
    T Lm = LP.mass - LP.invmass * P.invmass * P.invmass;
    *Lmass = sigma * Lm;
    for (int k = 0; k < 6; k++) {
        *Lmass += beta[k] * LIp[k];
        LI[k] = sigma * LIp[k];
    }
}

// Quaternion product a (x) b.
template <class T>
PG_HD void qmul4(const T a[4], const T b[4], T o[4]) {
    o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}
template <class T>
PG_HD void qaxis4(int axis, T ang, T o[4]) {
    T s = p_sin(ang * T(0.5f));
    o[0] = p_cos(ang * T(0.5f)); o[1] = o[2] = o[3] = T(0);
    o[1 + axis] = s;
}

// Release (src/sim.cu:79-107) with the pieces its adjoint needs: wb1 = rates + invI' (m' L1).
template <class T>
PG_HD St<T> release(const T* sc, const FlightP<T>& P, V3<T> cg, V3<T>* L1_out, V3<T>* wb1_out) {
    St<T> s;
    s.pos = v3(T(0), T(0), sc[SC_HEIGHT]);
    T qy[4], qp[4], qr[4], t1[4], q[4];
    qaxis4(2, sc[SC_YAW], qy);
    qaxis4(1, -sc[SC_PITCH], qp);
    qaxis4(0, sc[SC_ROLL], qr);
    qmul4(qp, qr, t1);
    qmul4(qy, t1, q);
    T l = p_sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int k = 0; k < 4; k++) s.q[k] = q[k] / l;
    T fy[4], fp[4], qf[4];
    qaxis4(2, sc[SC_YAW] + sc[SC_FY], fy);
    qaxis4(1, -(sc[SC_PITCH] + sc[SC_FP]), fp);
    qmul4(fy, fp, qf);
    M3<T> Rf;
    rot_rows(qf, Rf);
    s.vel = v3(Rf.a[0][0] * sc[SC_SPEED], Rf.a[1][0] * sc[SC_SPEED], Rf.a[2][0] * sc[SC_SPEED]);
    M3<T> R;
    rot_rows(s.q, R);
    V3<T> vb;
    for (int j = 0; j < 3; j++) (&vb.x)[j] = R.a[0][j] * s.vel.x + R.a[1][j] * s.vel.y + R.a[2][j] * s.vel.z;
    V3<T> grip = v3(sc[SC_GX], sc[SC_GY], sc[SC_GZ]);
    V3<T> L1 = cross(grip - cg, vb) * T(0.12f);  // per unit mass
    V3<T> mL = L1 * P.mass;
    V3<T> wb1 = v3(sc[SC_RR] + P.invI[0] * mL.x + P.invI[1] * mL.y + P.invI[2] * mL.z,
                   sc[SC_PR] + P.invI[3] * mL.x + P.invI[4] * mL.y + P.invI[5] * mL.z,
                   sc[SC_YR] + P.invI[6] * mL.x + P.invI[7] * mL.y + P.invI[8] * mL.z);
    s.w = clamp_len(wb1, T(35));
    s.t = T(0);
    if (L1_out) *L1_out = L1;
    if (wb1_out) *wb1_out = wb1;
    return s;
}
template <class T>
PG_HD void release_adj(const FlightP<T>& P, V3<T> L1, V3<T> wb1, const St<T>& L0, LamP<T>& LP) {
    V3<T> Lwb1 = clamp_len_adj(wb1, T(35), L0.w);
    V3<T> mL = L1 * P.mass;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) LP.invI[r * 3 + c] += (&Lwb1.x)[r] * (&mL.x)[c];
    V3<T> iL = v3(P.invI[0] * L1.x + P.invI[1] * L1.y + P.invI[2] * L1.z,
                  P.invI[3] * L1.x + P.invI[4] * L1.y + P.invI[5] * L1.z,
                  P.invI[6] * L1.x + P.invI[7] * L1.y + P.invI[8] * L1.z);
    LP.mass += dot(Lwb1, iL);
}

// Staging of one panel (print-warped normal, CG shift, dynamic-pressure area) and its adjoint.
template <class T>
PG_HD void stage(V3<T> c, T A, V3<T> n, V3<T> cg, T rho, T wp, T wr, V3<T>* rb, V3<T>* nb, T* ak) {
    *rb = c - cg;
    T ar = wr * p_max(T(-1), p_min(T(1), rb->y * T(8)));
    T ap = wp * p_max(T(-1), p_min(T(1), rb->x * T(8)));
    V3<T> nr = v3(n.x, n.y - ar * n.z, n.z + ar * n.y);
    V3<T> nu = v3(nr.x + ap * nr.z, nr.y, nr.z - ap * nr.x);
    T l = p_sqrt(dot(nu, nu));
    *nb = l > T(1e-12f) ? nu * (T(1) / l) : v3(T(0), T(0), T(1));
    *ak = T(0.5f) * rho * A;
}
template <class T>
PG_HD void stage_adj(V3<T> c, V3<T> n, V3<T> cg, T rho, T wp, T wr, V3<T> Lrb, V3<T> Lnb, T Lak, V3<T>* Lc,
                     T* LA, V3<T>* Ln) {
    V3<T> rb = c - cg;
    T cy = rb.y * T(8), cx = rb.x * T(8);
    T ar = wr * p_max(T(-1), p_min(T(1), cy));
    T ap = wp * p_max(T(-1), p_min(T(1), cx));
    V3<T> nr = v3(n.x, n.y - ar * n.z, n.z + ar * n.y);
    V3<T> nu = v3(nr.x + ap * nr.z, nr.y, nr.z - ap * nr.x);
    T l = p_sqrt(dot(nu, nu));
    *LA = T(0.5f) * rho * Lak;
    V3<T> Lrbt = Lrb;
    if (l > T(1e-12f)) {
        V3<T> nb = nu * (T(1) / l);
        V3<T> Lnu = (Lnb - nb * dot(nb, Lnb)) * (T(1) / l);
        V3<T> Lnr = v3(Lnu.x - ap * Lnu.z, Lnu.y, ap * Lnu.x + Lnu.z);
        T Lap = Lnu.x * nr.z - Lnu.z * nr.x;
        *Ln = v3(Lnr.x, Lnr.y + ar * Lnr.z, -ar * Lnr.y + Lnr.z);
        T Lar = -Lnr.y * n.z + Lnr.z * n.y;
        if (cy > T(-1) && cy < T(1)) Lrbt.y += Lar * wr * T(8);
        if (cx > T(-1) && cx < T(1)) Lrbt.x += Lap * wp * T(8);
    } else {
        *Ln = v3(T(0), T(0), T(0));
    }
    *Lc = Lrbt;
}

// Tail-aware weights dJ/dd_s of 0.65 mean + 0.25 mean(worst ceil(S/4)) + 0.10 min.
template <class T>
PG_HD T objective_weights(const T* d, int S, T* w) {
    int tail = (S + 3) / 4;
    T mean = T(0);
    for (int s = 0; s < S; s++) { mean += d[s] / T(S); w[s] = T(0.65) / T(S); }
    // rank by (value, index): selection of the tail without sorting
    T cvar = T(0), mn = d[0];
    int imin = 0;
    for (int s = 0; s < S; s++) {
        int rank = 0;
        for (int k = 0; k < S; k++) rank += (d[k] < d[s]) || (d[k] == d[s] && k < s);
        if (rank < tail) { w[s] += T(0.25) / T(tail); cvar += d[s] / T(tail); }
        if (d[s] < mn) { mn = d[s]; imin = s; }
    }
    w[imin] += T(0.10);
    return T(0.65) * mean + T(0.25) * cvar + T(0.10) * mn;
}


// ------------------------------------------------------------------ whole-flight gradient (serial form)
// The serial form of the per-flight reverse pass, used by host tests; the GPU kernel runs the
// same pieces with the panel loops spread over lanes.
template <class T>
struct PlaneData {  // what mass_props and the panel pass give a flight
    T mass, I[6];
    int nt;
    V3<T> c[kNtMax];
    T A[kNtMax];
    V3<T> n[kNtMax];
};
template <class T>
struct PlaneAdj {  // adjoint of a flight's distance wrt that plane data
    T mass, I[6];
    V3<T> c[kNtMax];
    T A[kNtMax];
    V3<T> n[kNtMax];
};

// Clock of the state before step j given the clock before step j-1 (the reference restarts the
// clock at every 600-step launch, src/sim.cu:113).
template <class T>
PG_HD T next_clock(T t, int j) { return (j % 600 == 0) ? T((double)j) * T(kDt) : t + T(kDt); }

template <class T>
T flight_grad_serial(const T* sc, T phase, const PlaneData<T>& pd, int max_steps, int K, PlaneAdj<T>& out,
                     int* kind_out, int* steps_out, St<T>* ck /* >= max_steps / K + 2 */) {
    FlightP<T> P;
    V3<T> cg;
    T sigma, beta[6];
    printed(sc, pd.mass, pd.I, P, &cg, &sigma, beta);
    P.phase = phase;
    static thread_local V3<T> rb[kNtMax], nb[kNtMax], Lrb[kNtMax], Lnb[kNtMax];
    static thread_local T ak[kNtMax], Lak[kNtMax];
    for (int i = 0; i < pd.nt; i++) {
        stage(pd.c[i], pd.A[i], pd.n[i], cg, sc[SC_RHO], sc[SC_WP], sc[SC_WR], &rb[i], &nb[i], &ak[i]);
        Lrb[i] = v3(T(0), T(0), T(0)); Lnb[i] = Lrb[i]; Lak[i] = T(0);
    }
    V3<T> L1rel, wb1;
    St<T> s = release(sc, P, cg, &L1rel, &wb1);
    // forward with checkpoints
    int k = -1, kind = 0;
    T d = T(0);
    St<T> before = s, after = s;
    for (int j = 0; j < max_steps; j++) {
        if (j > 0) s.t = next_clock(before.t, j);
        if (j % K == 0) ck[j / K] = s;
        Pre<T> pr;
        step_pre(P, s, pr);
        V3<T> Fb = v3(T(0), T(0), T(0)), Tb = Fb;
        for (int i = 0; i < pd.nt; i++) {
            V3<T> f, tq;
            panel_fwd(pr, rb[i], nb[i], ak[i], P.cf, &f, &tq);
            Fb = Fb + f; Tb = Tb + tq;
        }
        before = s;
        after = step_post(P, s, pr, Fb, Tb);
        if (terminate(before, after, j, max_steps, &d, &kind)) { k = j; break; }
        s = after;
    }
    *kind_out = kind;
    *steps_out = k + 1;
    out.mass = T(0);
    for (int q = 0; q < 6; q++) out.I[q] = T(0);
    for (int i = 0; i < pd.nt; i++) { out.c[i] = v3(T(0), T(0), T(0)); out.n[i] = out.c[i]; out.A[i] = T(0); }
    if (kind == 3 || k < 0) return d;
    // reverse sweep, segment by segment
    LamP<T> LP;
    LP.mass = LP.invmass = T(0);
    for (int q = 0; q < 6; q++) LP.I[q] = T(0);
    for (int q = 0; q < 9; q++) LP.invI[q] = T(0);
    St<T> Lnext, Lb;
    auto zero = [](St<T>& z) {
        z.pos = v3(T(0), T(0), T(0)); z.vel = z.pos; z.w = z.pos; z.q[0] = z.q[1] = z.q[2] = z.q[3] = T(0); z.t = T(0);
    };
    zero(Lnext); zero(Lb);
    terminate_adj(before, after, kind, Lb, Lnext);
    static thread_local St<T> seg[1024];
    for (int sg = k / K; sg >= 0; sg--) {
        int j0 = sg * K, j1 = (j0 + K - 1 < k) ? j0 + K - 1 : k;  // steps j0..j1
        seg[0] = ck[sg];
        for (int j = j0; j < j1; j++) {  // states before steps j0..j1
            St<T> cur = seg[j - j0];
            Pre<T> pr;
            step_pre(P, cur, pr);
            V3<T> Fb = v3(T(0), T(0), T(0)), Tb = Fb;
            for (int i = 0; i < pd.nt; i++) {
                V3<T> f, tq;
                panel_fwd(pr, rb[i], nb[i], ak[i], P.cf, &f, &tq);
                Fb = Fb + f; Tb = Tb + tq;
            }
            St<T> nx = step_post(P, cur, pr, Fb, Tb);
            nx.t = next_clock(cur.t, j + 1);
            seg[j - j0 + 1] = nx;
        }
        for (int j = j1; j >= j0; j--) {
            const St<T>& cur = seg[j - j0];
            Pre<T> pr;
            step_pre(P, cur, pr);
            V3<T> Fb = v3(T(0), T(0), T(0)), Tb = Fb;
            for (int i = 0; i < pd.nt; i++) {
                V3<T> f, tq;
                panel_fwd(pr, rb[i], nb[i], ak[i], P.cf, &f, &tq);
                Fb = Fb + f; Tb = Tb + tq;
            }
            St<T> L0;
            zero(L0);
            M3<T> LR;
            for (int a = 0; a < 3; a++) for (int b = 0; b < 3; b++) LR.a[a][b] = T(0);
            V3<T> LFb, LTb;
            step_post_adj(P, cur, pr, Fb, Tb, Lnext, L0, &LFb, &LTb, LR, LP);
            V3<T> Lvb = v3(T(0), T(0), T(0)), Lwp = Lvb;
            for (int i = 0; i < pd.nt; i++) panel_adj(pr, rb[i], nb[i], ak[i], P.cf, LFb, LTb, &Lrb[i], &Lnb[i], &Lak[i], &Lvb, &Lwp);
            step_pre_adj(P, cur, pr, Lvb, Lwp, LR, L0);
            if (j == k) {
                L0.pos = L0.pos + Lb.pos;
            }
            Lnext = L0;
        }
    }
    release_adj(P, L1rel, wb1, Lnext, LP);
    printed_adj(P, sigma, beta, LP, &out.mass, out.I);
    for (int i = 0; i < pd.nt; i++)
        stage_adj(pd.c[i], pd.n[i], cg, sc[SC_RHO], sc[SC_WP], sc[SC_WR], Lrb[i], Lnb[i], Lak[i], &out.c[i], &out.A[i],
                  &out.n[i]);
    return d;
}

// Plane data of a genome in scalar S (float, double or a dual number).
template <class S>
PG_HD void plane_data(const S* g, V3<S>* V, S* mass, S I[6], V3<S>* com, int* nt) {
    Topo tp = topology(g);
    for (int i = 0; i < tp.nv; i++) V[i] = mesh_vertex(g, tp, i);
    mass_props(g, V, tp, mass, com, I);
    *nt = tp.nt;
}

// dJ/dg_j = adjoint . d(plane data)/dg_j, by one dual-number pass through the mesh.
template <class T>
PG_HD T genome_jvp(const float* genome, int j, const PlaneAdj<T>& ybar, V3<Dual<T>>* Vbuf) {
    Dual<T> g[35];
    for (int k = 0; k < 35; k++) g[k] = Dual<T>(T(genome[k]), k == j ? T(1) : T(0));
    Dual<T> mass, I[6];
    V3<Dual<T>> com;
    int nt;
    plane_data(g, Vbuf, &mass, I, &com, &nt);
    Topo tp = topology(g);
    T acc = ybar.mass * mass.d;
    for (int q = 0; q < 6; q++) acc += ybar.I[q] * I[q].d;
    for (int t = 0; t < nt; t++) {
        V3<Dual<T>> ct, n;
        Dual<T> A;
        panel(Vbuf, tp, com, t, &ct, &A, &n);
        acc += ybar.c[t].x * ct.x.d + ybar.c[t].y * ct.y.d + ybar.c[t].z * ct.z.d + ybar.A[t] * A.d +
               ybar.n[t].x * n.x.d + ybar.n[t].y * n.y.d + ybar.n[t].z * n.z.d;
    }
    return acc;
}

}  // namespace pg
