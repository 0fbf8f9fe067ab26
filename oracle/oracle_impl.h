/*
 * oracle_impl.h -- precision-generic body of the oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Included by oracle_f32.c (R = float, P = orf_) and oracle_f64.c (R = double, P = ord_).
 * Every expression keeps the operand order of the reference so that, in float and built
 * without FP contraction, the results are bit-identical to the reference's host-compiled
 * src/common.h.  Citations are to files of the reference project.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(P, name)

#if R_IS_DOUBLE
#define SIN_(x) sin(x)
#define COS_(x) cos(x)
#define TAN_(x) tan(x)
#define SQRT_(x) sqrt(x)
#define FABS_(x) fabs(x)
#define FMIN_(a, b) fmin(a, b)
#define FMAX_(a, b) fmax(a, b)
#else
#define SIN_(x) sinf(x)
#define COS_(x) cosf(x)
#define TAN_(x) tanf(x)
#define SQRT_(x) sqrtf(x)
#define FABS_(x) fabsf(x)
#define FMIN_(a, b) fminf(a, b)
#define FMAX_(a, b) fmaxf(a, b)
#endif
/* model constants are the reference's float literals in both precisions */
#define K(c) ((R)(c))

/* mesh resolution and shell model, src/common.h:106-115 */
#define CH_ 5
#define SP_ 8
#define PLA_WALL_ 0.00045f
#define SHELL_RHO_ (1240.0f * 0.00045f)
#define PRINT_LIMIT_ (0.250f - 0.00045f)
/* flight constants, src/common.h:470-478 */
#define DT_ (1.0f / 600.0f)
#define CN_SLOPE_ 1.9f
#define GRAV_ 9.81f

typedef struct { R x, y, z; } v3r;
typedef struct { R w, x, y, z; } qr;

static inline v3r mk(R x, R y, R z) { v3r a; a.x = x; a.y = y; a.z = z; return a; }
static inline v3r vadd(v3r a, v3r b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3r vsub(v3r a, v3r b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3r vscl(v3r a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline R vdot(v3r a, v3r b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3r vcross(v3r a, v3r b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline R vlen(v3r a) { return SQRT_(vdot(a, a)); }
static inline v3r vnorm(v3r a) {
    R l = vlen(a);
    return l > K(1e-12f) ? vscl(a, K(1.0f) / l) : mk(0, 0, 1);
}
static inline qr mq(R w, R x, R y, R z) { qr q; q.w = w; q.x = x; q.y = y; q.z = z; return q; }
static inline qr qmul_(qr a, qr b) {
    return mq(a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z,
              a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
              a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
              a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w);
}
static inline qr qnorm_(qr q) {
    R l = SQRT_(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
    R il = K(1.0f) / l;
    return mq(q.w * il, q.x * il, q.y * il, q.z * il);
}
/* body->world rotation rows, src/common.h:38-43 */
static inline void qrows(qr q, v3r* r0, v3r* r1, v3r* r2) {
    R w = q.w, x = q.x, y = q.y, z = q.z;
    *r0 = mk(1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y));
    *r1 = mk(2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x));
    *r2 = mk(2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y));
}
static inline v3r qrot_(qr q, v3r v) {
    v3r r0, r1, r2; qrows(q, &r0, &r1, &r2);
    return mk(vdot(r0, v), vdot(r1, v), vdot(r2, v));
}
static inline v3r qrot_inv_(qr q, v3r v) {
    v3r r0, r1, r2; qrows(q, &r0, &r1, &r2);
    return mk(r0.x * v.x + r1.x * v.y + r2.x * v.z,
              r0.y * v.x + r1.y * v.y + r2.y * v.z,
              r0.z * v.x + r1.z * v.y + r2.z * v.z);
}
static inline qr qaxis_(v3r axis, R ang) {
    R s = SIN_(ang * K(0.5f)); v3r a = vnorm(axis);
    return mq(COS_(ang * K(0.5f)), a.x * s, a.y * s, a.z * s);
}

/* ---------------------------------------------------------------- genome view */
enum {
    G_SPAN, G_CHORD, G_TAPER, G_SWEEP, G_DIH_IN, G_DIH_OUT, G_KINK, G_CAMBER1, G_CAMBER2,
    G_WASHOUT, G_ELEVATOR, G_NOSE, G_KEEL, G_DECK_GAP, G_DECK_SCALE, G_BODY, G_FIN_H,
    G_FIN_CHORD, G_FIN_SWEEP, G_TAIL_SPAN, G_TAIL_CHORD, G_TAIL_ANGLE, G_LE_B1, G_LE_B2,
    G_CHORD_B1, G_CHORD_B2, G_FIN_LAYOUT, G_FIN_CANT, G_FIN_TAPER, G_FIN_SPAN_POS,
    G_TAIL_SWEEP, G_TAIL_TAPER, G_TAIL_DIH, G_TIP_ROUND, G_CENTER_CHORD
};
typedef struct { R v[35]; } gview;
static inline gview gload(const float* g) {
    gview o; for (int i = 0; i < 35; i++) o.v[i] = (R)g[i]; return o;
}
#define GV(g, f) ((g)->v[f])

/* ---------------------------------------------------------------- mesher */
/* src/common.h:124-129 */
static inline R camber(const gview* g, R xc) {
    R te = GV(g, G_ELEVATOR) * K(0.22f);
    R u = xc, v = K(1.0f) - u;
    return 3 * v * v * u * GV(g, G_CAMBER1) + 3 * v * u * u * GV(g, G_CAMBER2) + u * u * u * te;
}
/* src/common.h:132-141 */
static inline void spanyz(const gview* g, R t, R* y, R* z) {
    R half = GV(g, G_SPAN) * K(0.5f);
    R b = GV(g, G_BODY) * half, k = GV(g, G_KINK) * half;
    if (k < b) k = b;
    R yy = 0, zz = 0, seg;
    seg = FMIN_(t, b); yy += seg;
    seg = FMIN_(t, k) - b;
    if (seg > 0) { yy += seg * COS_(GV(g, G_DIH_IN)); zz += seg * SIN_(GV(g, G_DIH_IN)); }
    seg = t - k;
    if (seg > 0) { yy += seg * COS_(GV(g, G_DIH_OUT)); zz += seg * SIN_(GV(g, G_DIH_OUT)); }
    *y = yy; *z = zz;
}
/* src/common.h:144-172 */
static inline v3r wingpt(const gview* g, R u, R xc, R zoff, R scale) {
    R half = GV(g, G_SPAN) * K(0.5f) * scale;
    R t = FABS_(u) * half;
    R y, z; spanyz(g, t, &y, &z);
    R tf = FABS_(u);
    R v = K(1.0f) - tf;
    R cr = K(1.0f) + GV(g, G_CENTER_CHORD);
    R ct = GV(g, G_TAPER);
    R c1 = K(1.0f) + GV(g, G_CHORD_B1), c2 = ct + GV(g, G_CHORD_B2);
    R ratio = v * v * v * cr + 3 * v * v * tf * c1 + 3 * v * tf * tf * c2 + tf * tf * tf * ct;
    R ellipse = SQRT_(FMAX_(K(0.08f), K(1.0f) - K(0.92f) * tf * tf));
    ratio *= K(1.0f) - GV(g, G_TIP_ROUND) + GV(g, G_TIP_ROUND) * ellipse;
    ratio = FMAX_(K(0.035f), FMIN_(K(1.9f), ratio));
    R c = GV(g, G_CHORD) * scale * ratio;
    R xr = K(0.5f) * GV(g, G_CHORD) * scale * cr;
    R xt = K(0.5f) * GV(g, G_CHORD) * scale - TAN_(GV(g, G_SWEEP)) * half;
    R xb1 = xr + GV(g, G_LE_B1) * GV(g, G_CHORD) * scale;
    R xb2 = xt + GV(g, G_LE_B2) * GV(g, G_CHORD) * scale;
    R x_le = v * v * v * xr + 3 * v * v * tf * xb1 + 3 * v * tf * tf * xb2 + tf * tf * tf * xt;
    R x = x_le - xc * c;
    R zc = z * scale + camber(g, xc) * c;
    R x_c4 = x_le - K(0.25f) * c;
    R tw = GV(g, G_WASHOUT) * tf;
    zc += tw * (x - x_c4);
    return mk(x, (u < 0 ? -y : y), zc + zoff);
}

static inline void put_tri(int* T, int* nt, int a, int b, int c) {
    T[*nt * 3 + 0] = a; T[*nt * 3 + 1] = b; T[*nt * 3 + 2] = c; (*nt)++;
}
static inline void put_v(R* V, int* nv, v3r p) {
    V[*nv * 3 + 0] = p.x; V[*nv * 3 + 1] = p.y; V[*nv * 3 + 2] = p.z; (*nv)++;
}
static inline v3r get_v(const R* V, int i) { return mk(V[i * 3], V[i * 3 + 1], V[i * 3 + 2]); }

/* src/common.h:177-192 */
static void wing_grid(const gview* g, R* V, int* T, int* nv, int* nt, R zoff, R scale) {
    int base = *nv;
    for (int i = 0; i <= 2 * SP_; i++) {
        R u = (R)(i - SP_) / (R)SP_;
        for (int j = 0; j <= CH_; j++) {
            R xc = (R)j / (R)CH_;
            put_v(V, nv, wingpt(g, u, xc, zoff, scale));
        }
    }
    for (int i = 0; i < 2 * SP_; i++)
        for (int j = 0; j < CH_; j++) {
            int a = base + i * (CH_ + 1) + j, b = a + CH_ + 1;
            put_tri(T, nt, a, b, a + 1);
            put_tri(T, nt, b, b + 1, a + 1);
        }
}
/* src/common.h:197-213 */
static void fin(const gview* g, R* V, int* T, int* nv, int* nt, R y0, R z0, int side) {
    R fc = GV(g, G_CHORD) * GV(g, G_FIN_CHORD);
    R sweep = fc * GV(g, G_FIN_SWEEP);
    R xr = K(-0.32f) * GV(g, G_CHORD) - GV(g, G_TAIL_CHORD) * GV(g, G_CHORD) * K(0.82f);
    R tipc = fc * GV(g, G_FIN_TAPER);
    R cant = side == 0 ? K(0.0f) : GV(g, G_FIN_CANT);
    R ya = y0 + (R)side * SIN_(cant) * GV(g, G_FIN_H);
    R za = z0 + COS_(cant) * GV(g, G_FIN_H);
    int base = *nv;
    put_v(V, nv, mk(xr + K(0.5f) * fc, y0, z0));
    put_v(V, nv, mk(xr - K(0.5f) * fc, y0, z0));
    put_v(V, nv, mk(xr - sweep + K(0.5f) * tipc, ya, za));
    put_v(V, nv, mk(xr - sweep - K(0.5f) * tipc, ya, za));
    put_tri(T, nt, base, base + 1, base + 2);
    put_tri(T, nt, base + 1, base + 3, base + 2);
}
/* src/common.h:215-255 */
static void tail(const gview* g, R* V, int* T, int* nv, int* nt) {
    R hs = K(0.5f) * GV(g, G_SPAN) * GV(g, G_TAIL_SPAN);
    R hc = GV(g, G_CHORD) * GV(g, G_TAIL_CHORD);
    R x0 = K(-0.32f) * GV(g, G_CHORD);
    R z0 = camber(g, K(0.82f)) * GV(g, G_CHORD);
    int base = *nv;
    for (int i = 0; i < 3; i++) {
        R u = (R)(i - 1), au = FABS_(u);
        R tc = hc * (K(1.0f) + (GV(g, G_TAIL_TAPER) - K(1.0f)) * au);
        R xle = x0 - GV(g, G_TAIL_SWEEP) * hc * au;
        for (int j = 0; j < 3; j++) {
            R xc = K(0.5f) * (R)j;
            R x = xle - xc * tc;
            R z = z0 + GV(g, G_TAIL_ANGLE) * (x - xle) + au * hs * SIN_(GV(g, G_TAIL_DIH));
            put_v(V, nv, mk(x, u * hs * COS_(GV(g, G_TAIL_DIH)), z));
        }
    }
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            int a = base + i * 3 + j, b = a + 3;
            put_tri(T, nt, a, b, a + 1);
            put_tri(T, nt, b, b + 1, a + 1);
        }
    R yp = hs * GV(g, G_FIN_SPAN_POS) * COS_(GV(g, G_TAIL_DIH));
    R zp = z0 + hs * GV(g, G_FIN_SPAN_POS) * SIN_(GV(g, G_TAIL_DIH));
    R layout = GV(g, G_FIN_LAYOUT);
    if (layout < K(0.25f)) {
        fin(g, V, T, nv, nt, 0, z0, 0);
    } else if (layout < K(0.50f)) {
        fin(g, V, T, nv, nt, -yp, zp, -1);
        fin(g, V, T, nv, nt, yp, zp, 1);
    } else if (layout < K(0.75f)) {
        fin(g, V, T, nv, nt, 0, z0, 0);
        fin(g, V, T, nv, nt, -yp, zp, -1);
        fin(g, V, T, nv, nt, yp, zp, 1);
    } else {
        R yo = hs * K(0.94f) * COS_(GV(g, G_TAIL_DIH));
        R zo = z0 + hs * K(0.94f) * SIN_(GV(g, G_TAIL_DIH));
        fin(g, V, T, nv, nt, -yo, zo, -1);
        fin(g, V, T, nv, nt, yo, zo, 1);
    }
}

/* src/common.h:257-292 */
int FN(build_mesh)(const float* genome, R* V, int* T, int* nv_out, int* nt_out) {
    gview gg = gload(genome); const gview* g = &gg;
    int nv = 0, nt = 0;
    wing_grid(g, V, T, &nv, &nt, 0, K(1.0f));
    tail(g, V, T, &nv, &nt);
    int decks = GV(g, G_DECK_GAP) > K(0.02f) ? 2 : 1;
    if (decks == 2) wing_grid(g, V, T, &nv, &nt, GV(g, G_DECK_GAP), GV(g, G_DECK_SCALE));
    {
        int base = nv;
        for (int j = 0; j <= 3; j++) {
            R xc = (R)j / (R)3;
            v3r top = wingpt(g, 0, xc, 0, K(1.0f));
            put_v(V, &nv, top);
            put_v(V, &nv, mk(top.x, 0, top.z - GV(g, G_KEEL) * (K(0.35f) + K(0.65f) * xc)));
        }
        for (int j = 0; j < 3; j++) {
            int a = base + j * 2;
            put_tri(T, &nt, a, a + 1, a + 2);
            put_tri(T, &nt, a + 1, a + 3, a + 2);
        }
    }
    if (decks == 2) {
        for (int s = -1; s <= 1; s += 2) {
            R u = (R)s * GV(g, G_KINK);
            int base = nv;
            v3r lo0 = wingpt(g, u, K(0.25f), 0, K(1.0f)), lo1 = wingpt(g, u, K(0.55f), 0, K(1.0f));
            v3r hi0 = wingpt(g, u * K(1.0f), K(0.25f), GV(g, G_DECK_GAP), GV(g, G_DECK_SCALE));
            v3r hi1 = wingpt(g, u * K(1.0f), K(0.55f), GV(g, G_DECK_GAP), GV(g, G_DECK_SCALE));
            put_v(V, &nv, lo0); put_v(V, &nv, lo1); put_v(V, &nv, hi0); put_v(V, &nv, hi1);
            put_tri(T, &nt, base, base + 1, base + 2);
            put_tri(T, &nt, base + 1, base + 3, base + 2);
        }
    }
    *nv_out = nv; *nt_out = nt;
    return 0;
}

/* src/common.h:294-307 */
void FN(mesh_extent)(const R* V, int nv, R* ext) {
    if (nv <= 0) { ext[0] = ext[1] = ext[2] = 0; return; }
    v3r lo = get_v(V, 0), hi = get_v(V, 0);
    for (int i = 1; i < nv; i++) {
        v3r p = get_v(V, i);
        lo.x = FMIN_(lo.x, p.x); lo.y = FMIN_(lo.y, p.y); lo.z = FMIN_(lo.z, p.z);
        hi.x = FMAX_(hi.x, p.x); hi.y = FMAX_(hi.y, p.y); hi.z = FMAX_(hi.z, p.z);
    }
    v3r e = vsub(hi, lo);
    ext[0] = e.x; ext[1] = e.y; ext[2] = e.z;
}
int FN(fits_print_volume)(const R* V, int nv) {
    R e[3]; FN(mesh_extent)(V, nv, e);
    R lim = K(PRINT_LIMIT_);
    return e[0] <= lim && e[1] <= lim && e[2] <= lim;
}

/* src/common.h:311-365 */
void FN(mass_props)(const float* genome, const R* V, const int* T, int nt, R* mp) {
    R chord = (R)genome[G_CHORD], nose = (R)genome[G_NOSE];
    R m = 0; v3r c = mk(0, 0, 0);
    for (int i = 0; i < nt; i++) {
        v3r a = get_v(V, T[i * 3]), b = get_v(V, T[i * 3 + 1]), d = get_v(V, T[i * 3 + 2]);
        R A = K(0.5f) * vlen(vcross(vsub(b, a), vsub(d, a)));
        R mi = A * K(SHELL_RHO_);
        v3r ct = vscl(vadd(vadd(a, b), d), K(1.0f / 3));
        m += mi; c = vadd(c, vscl(ct, mi));
    }
    R shell_m = m;
    v3r np = mk(K(0.5f) * chord, 0, 0);
    R mn = nose * shell_m;
    m += mn; c = vadd(c, vscl(np, mn));
    c = vscl(c, K(1.0f) / m);
    R I[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < nt; i++) {
        v3r a = get_v(V, T[i * 3]), b = get_v(V, T[i * 3 + 1]), d = get_v(V, T[i * 3 + 2]);
        R A = K(0.5f) * vlen(vcross(vsub(b, a), vsub(d, a)));
        R mi = A * K(SHELL_RHO_);
        v3r ra = vsub(a, c), rb = vsub(b, c), rd = vsub(d, c);
        R exx = (ra.x * ra.x + rb.x * rb.x + rd.x * rd.x + ra.x * rb.x + ra.x * rd.x + rb.x * rd.x) / K(6.0f);
        R eyy = (ra.y * ra.y + rb.y * rb.y + rd.y * rd.y + ra.y * rb.y + ra.y * rd.y + rb.y * rd.y) / K(6.0f);
        R ezz = (ra.z * ra.z + rb.z * rb.z + rd.z * rd.z + ra.z * rb.z + ra.z * rd.z + rb.z * rd.z) / K(6.0f);
        R exy = (2 * (ra.x * ra.y + rb.x * rb.y + rd.x * rd.y) +
                 ra.x * rb.y + rb.x * ra.y + ra.x * rd.y + rd.x * ra.y + rb.x * rd.y + rd.x * rb.y) / K(12.0f);
        R exz = (2 * (ra.x * ra.z + rb.x * rb.z + rd.x * rd.z) +
                 ra.x * rb.z + rb.x * ra.z + ra.x * rd.z + rd.x * ra.z + rb.x * rd.z + rd.x * rb.z) / K(12.0f);
        R eyz = (2 * (ra.y * ra.z + rb.y * rb.z + rd.y * rd.z) +
                 ra.y * rb.z + rb.y * ra.z + ra.y * rd.z + rd.y * ra.z + rb.y * rd.z + rd.y * rb.z) / K(12.0f);
        I[0] += mi * (eyy + ezz); I[1] += mi * (exx + ezz); I[2] += mi * (exx + eyy);
        I[3] -= mi * exy; I[4] -= mi * exz; I[5] -= mi * eyz;
        v3r nn = vnorm(vcross(vsub(b, a), vsub(d, a)));
        R th = mi * K(PLA_WALL_) * K(PLA_WALL_) / K(12.0f);
        I[0] += th * (K(1.0f) - nn.x * nn.x); I[1] += th * (K(1.0f) - nn.y * nn.y);
        I[2] += th * (K(1.0f) - nn.z * nn.z);
        I[3] -= th * nn.x * nn.y; I[4] -= th * nn.x * nn.z; I[5] -= th * nn.y * nn.z;
    }
    {
        v3r r = vsub(np, c);
        I[0] += mn * (r.y * r.y + r.z * r.z); I[1] += mn * (r.x * r.x + r.z * r.z);
        I[2] += mn * (r.x * r.x + r.y * r.y); I[3] -= mn * r.x * r.y;
        I[4] -= mn * r.x * r.z; I[5] -= mn * r.y * r.z;
    }
    R reg = K(1e-9f);
    R xx = I[0] + reg, yy = I[1] + reg, zz = I[2] + reg, xy = I[3], xz = I[4], yz = I[5];
    R det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
    R id = K(1.0f) / det;
    R* iv = mp + 11;
    iv[0] = (yy * zz - yz * yz) * id; iv[1] = (xz * yz - xy * zz) * id; iv[2] = (xy * yz - xz * yy) * id;
    iv[3] = iv[1]; iv[4] = (xx * zz - xz * xz) * id; iv[5] = (xy * xz - xx * yz) * id;
    iv[6] = iv[2]; iv[7] = iv[5]; iv[8] = (xx * yy - xy * xy) * id;
    mp[5] = xx; mp[6] = yy; mp[7] = zz; mp[8] = xy; mp[9] = xz; mp[10] = yz;
    mp[0] = m; mp[1] = K(1.0f) / m; mp[2] = c.x; mp[3] = c.y; mp[4] = c.z;
}

/* ---------------------------------------------------------------- scenarios */
/* src/common.h:368-375 */
static inline uint32_t mixb(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
static inline R su01(int seed, int lane) {
    return (R)(mixb((uint32_t)seed * 0x9e3779b9u + (uint32_t)lane * 0x85ebca6bu) >> 8) * K(1.0f / 16777216.0f);
}
static inline R ssgn(int seed, int lane) { return su01(seed, lane) * K(2.0f) - K(1.0f); }
/* (float)(seed * 37 % 97) with the two's-complement wrap of the 32-bit product */
static inline R seed_phase(int seed) {
    int32_t prod = (int32_t)((uint32_t)seed * 37u);
    return (R)(prod % 97);
}

/* src/common.h:389-421 */
void FN(scenario_desc)(int seed, R* d) {
    d[0] = K(9.2f) + K(2.0f) * ssgn(seed, 0);
    d[1] = K(0.10f) + K(0.20f) * ssgn(seed, 1);
    d[2] = K(0.12f) * ssgn(seed, 2);
    d[3] = K(0.16f) * ssgn(seed, 3);
    d[4] = K(1.75f) + K(0.35f) * ssgn(seed, 4);
    d[5] = K(1.8f) * ssgn(seed, 5);
    d[6] = K(1.2f) * ssgn(seed, 6);
    d[7] = K(1.5f) * ssgn(seed, 7);
    d[8] = K(1.225f) * (K(0.88f) + K(0.22f) * su01(seed, 8));
    d[9] = K(0.02f) * (K(0.75f) + K(0.55f) * su01(seed, 9));
    d[10] = K(0.45f) + K(1.10f) * (K(0.5f) + K(0.5f) * SIN_((R)seed * K(1.61803f)));
    R phase = seed_phase(seed);
    d[11] = K(-0.25f) + K(1.15f) * SIN_(phase * K(0.71f));
    d[12] = K(1.00f) * SIN_(phase * K(1.13f));
    d[13] = K(0.075f) * ssgn(seed, 10);
    d[14] = K(0.060f) * ssgn(seed, 11);
    d[15] = K(0.018f) * ssgn(seed, 12);
    d[16] = K(0.022f) * ssgn(seed, 13);
    d[17] = K(0.010f) * ssgn(seed, 14);
    d[18] = K(0.88f) + K(0.24f) * su01(seed, 15);
    d[19] = K(0.06f) + K(0.34f) * su01(seed, 16);
    d[20] = K(0.018f) * ssgn(seed, 17);
    d[21] = K(0.010f) * ssgn(seed, 18);
    d[22] = K(0.006f) * ssgn(seed, 19);
    d[9] *= K(0.90f) + K(0.25f) * su01(seed, 20);
    d[23] = K(0.025f) * ssgn(seed, 21);
    d[24] = K(0.035f) * ssgn(seed, 22);
}

/* src/common.h:423-427 */
static inline void pt_inertia(R I[6], v3r r, R m) {
    I[0] += m * (r.y * r.y + r.z * r.z); I[1] += m * (r.x * r.x + r.z * r.z);
    I[2] += m * (r.x * r.x + r.y * r.y); I[3] -= m * r.x * r.y;
    I[4] -= m * r.x * r.z; I[5] -= m * r.y * r.z;
}
/* src/common.h:429-436 (inverse into mp[11..19] from mp[5..10]) */
static inline void inv_inertia(R* mp) {
    R xx = mp[5], yy = mp[6], zz = mp[7], xy = mp[8], xz = mp[9], yz = mp[10];
    R det = xx * (yy * zz - yz * yz) - xy * (xy * zz - yz * xz) + xz * (xy * yz - yy * xz);
    R id = K(1.0f) / FMAX_(det, K(1e-24f));
    R* iv = mp + 11;
    iv[0] = (yy * zz - yz * yz) * id; iv[1] = (xz * yz - xy * zz) * id; iv[2] = (xy * yz - xz * yy) * id;
    iv[3] = iv[1]; iv[4] = (xx * zz - xz * xz) * id; iv[5] = (xy * xz - xx * yz) * id;
    iv[6] = iv[2]; iv[7] = iv[5]; iv[8] = (xx * yy - xy * xy) * id;
}
/* src/common.h:441-457 */
void FN(printed_mass_props)(const R* src, const R* d, R* out, R* cg_out) {
    R mp[20]; memcpy(mp, src, sizeof mp);
    R m_shell = mp[0] * d[18];
    R m_fill = m_shell * d[19];
    R m = m_shell + m_fill;
    v3r bias = mk(d[20], d[21], d[22]);
    v3r cg = vscl(bias, m_fill / m);
    R scale = m / mp[0];
    for (int k = 0; k < 6; k++) mp[5 + k] *= scale;
    pt_inertia(mp + 5, vscl(cg, K(-1.0f)), m_shell);
    pt_inertia(mp + 5, vsub(bias, cg), m_fill);
    mp[0] = m; mp[1] = K(1.0f) / m;
    mp[2] = mp[2] + cg.x; mp[3] = mp[3] + cg.y; mp[4] = mp[4] + cg.z;
    inv_inertia(mp);
    memcpy(out, mp, sizeof mp);
    cg_out[0] = cg.x; cg_out[1] = cg.y; cg_out[2] = cg.z;
}

/* src/common.h:459-467 */
static inline v3r wind(v3r p, R t, int seed, R gust, R base_x, R base_y) {
    R s = seed_phase(seed);
    R gx = gust * (K(0.55f) * SIN_(K(0.9f) * p.x + K(1.3f) * t + s) +
                   K(0.35f) * SIN_(K(2.3f) * p.z + K(2.1f) * t + K(1.7f) * s) +
                   K(0.25f) * SIN_(K(4.1f) * p.y + K(3.3f) * t + K(0.4f) * s));
    R gy = gust * (K(0.50f) * SIN_(K(1.1f) * p.x + K(1.7f) * t + K(2.2f) * s) +
                   K(0.30f) * SIN_(K(3.1f) * p.z + K(2.9f) * t + K(0.9f) * s));
    R gz = gust * (K(0.30f) * SIN_(K(1.4f) * p.x + K(2.3f) * t + K(3.1f) * s) +
                   K(0.20f) * SIN_(K(2.7f) * p.y + K(1.9f) * t + K(1.2f) * s));
    return mk(base_x + gx, base_y + gy, gz);
}
void FN(wind_at)(const R* p, R t, int seed, R* out) {
    R d[25]; FN(scenario_desc)(seed, d);
    v3r w = wind(mk(p[0], p[1], p[2]), t, seed, d[10], d[11], d[12]);
    out[0] = w.x; out[1] = w.y; out[2] = w.z;
}

/* ---------------------------------------------------------------- prepare (src/sim.cu:25-49) */
void FN(prepare)(const float* genomes, int pop, R* pc, R* pn, R* mpo, int* nto) {
    R* V = (R*)malloc(sizeof(R) * OR_MAX_V * 3);
    int* T = (int*)malloc(sizeof(int) * OR_MAX_T * 3);
    for (int i = 0; i < pop; i++) {
        const float* g = genomes + (size_t)i * OR_GENOME_N;
        int nv, nt;
        FN(build_mesh)(g, V, T, &nv, &nt);
        R* mp = mpo + (size_t)i * OR_MP_N;
        FN(mass_props)(g, V, T, nt, mp);
        int printable = FN(fits_print_volume)(V, nv);
        int ntp = printable ? nt : 0;
        nto[i] = ntp;
        v3r com = mk(mp[2], mp[3], mp[4]);
        for (int t = 0; t < ntp; t++) {
            v3r a = vsub(get_v(V, T[t * 3]), com), b = vsub(get_v(V, T[t * 3 + 1]), com);
            v3r c = vsub(get_v(V, T[t * 3 + 2]), com);
            v3r nrm = vcross(vsub(b, a), vsub(c, a));
            R A = K(0.5f) * vlen(nrm);
            v3r ct = vscl(vadd(vadd(a, b), c), K(1.0f / 3));
            R* o = pc + ((size_t)i * OR_MAX_T + t) * 4;
            o[0] = ct.x; o[1] = ct.y; o[2] = ct.z; o[3] = A;
            v3r n = A > K(1e-12f) ? vscl(nrm, K(0.5f) / A) : mk(0, 0, 1);
            R* q = pn + ((size_t)i * OR_MAX_T + t) * 4;
            q[0] = n.x; q[1] = n.y; q[2] = n.z; q[3] = 0;
        }
    }
    free(V); free(T);
}

/* ---------------------------------------------------------------- flight (src/sim.cu:55-212) */
typedef struct {
    R mp[20];      /* printed mass props */
    v3r cg;        /* print-bias CG shift */
    R env[25];     /* scenario */
    int seed;
} flight_ctx;

static void make_ctx(const R* mp_plane, int env_seed, flight_ctx* fc) {
    FN(scenario_desc)(env_seed, fc->env);
    R cg[3];
    FN(printed_mass_props)(mp_plane, fc->env, fc->mp, cg);
    fc->cg = mk(cg[0], cg[1], cg[2]);
    fc->seed = env_seed;
}

/* release, src/sim.cu:68-109, at the showcase grid offset (ox, oy, oz) (all 0 for the GA) */
static void do_release_at(const flight_ctx* fc, int nt, R* st, R ox, R oy, R oz) {
    const R* e = fc->env;
    R speed = e[0], pitch = e[1], yaw = e[2], roll = e[3], height = e[4];
    v3r pos = mk(ox, oy, height + oz);
    qr qyaw = qaxis_(mk(0, 0, 1), yaw);
    qr qpitch = qaxis_(mk(0, 1, 0), -pitch);
    qr qroll = qaxis_(mk(1, 0, 0), roll);
    qr q = qnorm_(qmul_(qyaw, qmul_(qpitch, qroll)));
    qr qfyaw = qaxis_(mk(0, 0, 1), yaw + e[14]);
    qr qfpitch = qaxis_(mk(0, 1, 0), -(pitch + e[13]));
    v3r vel = qrot_(qmul_(qfyaw, qfpitch), mk(speed, 0, 0));
    v3r wb = mk(e[5], e[6], e[7]);
    v3r grip = mk(e[15], e[16], e[17]);
    v3r Jb = qrot_inv_(q, vscl(vel, fc->mp[0]));
    v3r L = vscl(vcross(vsub(grip, fc->cg), Jb), K(0.12f));
    const R* iv = fc->mp + 11;
    v3r dwr = mk(iv[0] * L.x + iv[1] * L.y + iv[2] * L.z,
                 iv[3] * L.x + iv[4] * L.y + iv[5] * L.z,
                 iv[6] * L.x + iv[7] * L.y + iv[8] * L.z);
    wb = vadd(wb, dwr);
    R w0 = vlen(wb);
    if (w0 > K(35.0f)) wb = vscl(wb, K(35.0f) / w0);
    st[0] = pos.x; st[1] = pos.y; st[2] = pos.z;
    st[3] = q.w; st[4] = q.x; st[5] = q.y; st[6] = q.z;
    st[7] = vel.x; st[8] = vel.y; st[9] = vel.z;
    st[10] = wb.x; st[11] = wb.y; st[12] = wb.z;
    st[13] = 0; st[14] = nt <= 0 ? K(1.0f) : K(0.0f); st[15] = nt <= 0 ? K(-100.0f) : K(0.0f);
}

static void do_release(const flight_ctx* fc, int nt, R* st) { do_release_at(fc, nt, st, 0, 0, 0); }

void FN(release)(const R* mp_plane, int nt, int env_seed, R* state) {
    flight_ctx fc; make_ctx(mp_plane, env_seed, &fc);
    do_release(&fc, nt, state);
}

/* One 600 Hz step from st (src/sim.cu:129-204).  The aerodynamic sums follow k_sim's order:
 * 128 threads with strided panels, a 5-level shuffle tree per warp, then a serial 4-warp sum.
 * Returns 1 when the flight ended at this step.  FT (optional) receives the aerodynamic
 * force and torque sums (world frame, gravity excluded). */
static int do_step(const flight_ctx* fc, const R* pc, const R* pn, int nt, R* st, int step,
                   int max_steps, R* FT) {
    const R* e = fc->env;
    v3r pos = mk(st[0], st[1], st[2]);
    qr q = mq(st[3], st[4], st[5], st[6]);
    v3r vel = mk(st[7], st[8], st[9]), wb = mk(st[10], st[11], st[12]);
    R t = st[13];
    v3r r0, r1, r2; qrows(q, &r0, &r1, &r2);
    v3r ww = mk(vdot(r0, wb), vdot(r1, wb), vdot(r2, wb));
    v3r wnd = wind(pos, t, fc->seed, e[10], e[11], e[12]);
    R acc[128][6];
    memset(acc, 0, sizeof acc);
    R air_rho = e[8], skin_cf = e[9], warp_pitch = e[23], warp_roll = e[24];
    for (int i = 0; i < nt; i++) {
        const R* c4 = pc + (size_t)i * 4; const R* n4 = pn + (size_t)i * 4;
        v3r rb = vsub(mk(c4[0], c4[1], c4[2]), fc->cg); R A = c4[3];
        v3r nb = mk(n4[0], n4[1], n4[2]);
        R ar = warp_roll * FMAX_(K(-1.f), FMIN_(K(1.f), rb.y / K(0.125f)));
        R ap = warp_pitch * FMAX_(K(-1.f), FMIN_(K(1.f), rb.x / K(0.125f)));
        v3r nr = mk(nb.x, nb.y - ar * nb.z, nb.z + ar * nb.y);
        nb = vnorm(mk(nr.x + ap * nr.z, nr.y, nr.z - ap * nr.x));
        v3r rw = mk(vdot(r0, rb), vdot(r1, rb), vdot(r2, rb));
        v3r nw = mk(vdot(r0, nb), vdot(r1, nb), vdot(r2, nb));
        v3r vr = vsub(vadd(vel, vcross(ww, rw)), wnd);
        R V2 = vdot(vr, vr);
        if (V2 < K(1e-6f)) continue;
        R Vm = SQRT_(V2);
        v3r vh = vscl(vr, K(1.0f) / Vm);
        R s = vdot(vh, nw);
        R qd = K(0.5f) * air_rho * V2 * A;
        R cn = K(CN_SLOPE_) * s * SQRT_(FMAX_(K(0.f), K(1.f) - s * s)) + K(2.0f) * s * FABS_(s);
        v3r f = vscl(nw, -qd * cn);
        v3r tang = vsub(vh, vscl(nw, s));
        f = vsub(f, vscl(tang, qd * skin_cf));
        v3r tq = vcross(rw, f);
        R* a = acc[i & 127];
        a[0] = a[0] + f.x; a[1] = a[1] + f.y; a[2] = a[2] + f.z;
        a[3] = a[3] + tq.x; a[4] = a[4] + tq.y; a[5] = a[5] + tq.z;
    }
    R sum[6] = {0, 0, 0, 0, 0, 0};
    for (int w = 0; w < 4; w++) {
        R lane[32][6];
        memcpy(lane, acc[w * 32], sizeof lane);
        for (int o = 16; o > 0; o >>= 1)
            for (int l = 0; l < o; l++)
                for (int k = 0; k < 6; k++) lane[l][k] = lane[l][k] + lane[l + o][k];
        for (int k = 0; k < 6; k++) sum[k] = sum[k] + lane[0][k];
    }
    if (FT) for (int k = 0; k < 6; k++) FT[k] = sum[k];
    const R* mp = fc->mp;
    v3r Fs = mk(sum[0], sum[1], sum[2]), Ts = mk(sum[3], sum[4], sum[5]);
    Fs.z -= mp[0] * K(GRAV_);
    v3r tb = mk(r0.x * Ts.x + r1.x * Ts.y + r2.x * Ts.z,
                r0.y * Ts.x + r1.y * Ts.y + r2.y * Ts.z,
                r0.z * Ts.x + r1.z * Ts.y + r2.z * Ts.z);
    const R* I = mp + 5; const R* iv = mp + 11;
    v3r Iw = mk(I[0] * wb.x + I[3] * wb.y + I[4] * wb.z,
                I[3] * wb.x + I[1] * wb.y + I[5] * wb.z,
                I[4] * wb.x + I[5] * wb.y + I[2] * wb.z);
    v3r gyro = vcross(wb, Iw);
    v3r tqb = vsub(tb, gyro);
    v3r dw = mk(iv[0] * tqb.x + iv[1] * tqb.y + iv[2] * tqb.z,
                iv[3] * tqb.x + iv[4] * tqb.y + iv[5] * tqb.z,
                iv[6] * tqb.x + iv[7] * tqb.y + iv[8] * tqb.z);
    wb = vadd(wb, vscl(dw, K(DT_)));
    R wl = vlen(wb);
    if (wl > K(150.f)) wb = vscl(wb, K(150.f) / wl);
    vel = vadd(vel, vscl(Fs, mp[1] * K(DT_)));
    R vl = vlen(vel);
    if (vl > K(60.f)) vel = vscl(vel, K(60.f) / vl);
    pos = vadd(pos, vscl(vel, K(DT_)));
    qr dq = qmul_(q, mq(0, wb.x, wb.y, wb.z));
    q = qnorm_(mq(q.w + K(0.5f) * dq.w * K(DT_), q.x + K(0.5f) * dq.x * K(DT_),
                  q.y + K(0.5f) * dq.y * K(DT_), q.z + K(0.5f) * dq.z * K(DT_)));
    t += K(DT_);
    st[0] = pos.x; st[1] = pos.y; st[2] = pos.z;
    st[3] = q.w; st[4] = q.x; st[5] = q.y; st[6] = q.z;
    st[7] = vel.x; st[8] = vel.y; st[9] = vel.z;
    st[10] = wb.x; st[11] = wb.y; st[12] = wb.z; st[13] = t;
    int bad = !(pos.x == pos.x && vel.x == vel.x);
    if (pos.z <= K(0.0f) || bad || FABS_(pos.y) > K(300.f) || pos.x < K(-50.f)) {
        st[14] = 1; st[15] = bad ? K(-10.0f) : pos.x; return 1;
    } else if (step == max_steps - 1) {
        st[14] = 1; st[15] = pos.x; return 1;
    }
    return 0;
}

void FN(step)(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed,
              const R* state_in, int step, int max_steps, R* state_out, R* FT) {
    flight_ctx fc; make_ctx(mp_plane, env_seed, &fc);
    memcpy(state_out, state_in, sizeof(R) * OR_STATE_N);
    do_step(&fc, pc, pn, nt, state_out, step, max_steps, FT);
}

/* A whole flight: the reference runs it as 600-step launches, each of which restarts its
 * clock at step0 * SIM_DT (src/sim.cu:113, 241-244); that reset is reproduced here. */
void FN(fly)(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed, int max_steps,
             R* fitness, int* steps, R* state_out) {
    flight_ctx fc; make_ctx(mp_plane, env_seed, &fc);
    R st[OR_STATE_N];
    do_release(&fc, nt, st);
    int n = 0;
    if (nt > 0) {
        for (int step = 0; step < max_steps; step++) {
            if (step > 0 && step % OR_CHUNK == 0) st[13] = (R)step * K(DT_);
            n = step + 1;
            if (do_step(&fc, pc, pn, nt, st, step, max_steps, NULL)) break;
        }
    }
    *fitness = st[15]; *steps = n;
    if (state_out) memcpy(state_out, st, sizeof st);
}

/* The landing distance interpolated between the last state above ground and the first at or
 * below it (continuous in the genome; the objective that gradients are checked on).  Flights
 * ended otherwise keep the reference's fitness.  kind: 0 oversize, 1 ground, 2 other, 3 NaN. */
void FN(fly_smooth)(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed, int max_steps,
                    R* d, int* steps, int* kind) {
    flight_ctx fc; make_ctx(mp_plane, env_seed, &fc);
    R st[OR_STATE_N];
    do_release(&fc, nt, st);
    *steps = 0; *kind = 0; *d = st[15];
    if (nt <= 0) return;
    for (int step = 0; step < max_steps; step++) {
        if (step > 0 && step % OR_CHUNK == 0) st[13] = (R)step * K(DT_);
        R x0 = st[0], z0 = st[2];
        *steps = step + 1;
        if (do_step(&fc, pc, pn, nt, st, step, max_steps, NULL)) {
            R x1 = st[0], z1 = st[2], vx = st[7];
            if (!(x1 == x1 && vx == vx)) { *d = K(-10.0f); *kind = 3; }
            else if (z1 <= 0) { *d = x0 + (x1 - x0) * (z0 / (z0 - z1)); *kind = 1; }
            else { *d = x1; *kind = 2; }
            return;
        }
    }
}

/* The reference's gpu_sim with pose recording and the showcase launch grid (src/sim.cu:72-79,
 * 115-128, 238-248): twelve 600-step launches; each starts its record index at step0 / rec_every
 * and, at every step that is a multiple of rec_every, writes (pos, q, alive) before integrating,
 * while the index is below rec_cap.  A finished flight keeps being recorded (alive 0) until step
 * 7199.  Plane p of a launch grid with spacing `spread` (> 0) starts at
 * ((p / 25) * -1.4 spread, (p % 25 - 12) spread, 0.25 sin(12.9898 p)) from the scenario's hand. */
void FN(fly_rec)(const R* pc, const R* pn, int nt, const R* mp_plane, int env_seed, int p, R spread,
                 int rec_every, int rec_cap, R* rec, R* fitness) {
    flight_ctx fc; make_ctx(mp_plane, env_seed, &fc);
    R st[OR_STATE_N];
    R ox = 0, oy = 0, oz = 0;
    if (spread > 0) {
        int cols = 25;
        oy = (R)((p % cols) - cols / 2) * spread;
        ox = -(R)(p / cols) * spread * K(1.4f);
        oz = K(0.25f) * SIN_((R)p * K(12.9898f));
    }
    do_release_at(&fc, nt, st, ox, oy, oz);
    for (int step0 = 0; step0 < OR_SIM_MAX_STEPS; step0 += OR_CHUNK) {
        if (step0 > 0) st[13] = (R)step0 * K(DT_);
        int rec_i = step0 / rec_every;
        for (int step = step0; step < step0 + OR_CHUNK; step++) {
            if (step % rec_every == 0 && rec_i < rec_cap) {
                R* r = rec + (size_t)rec_i * 8;
                r[0] = st[0]; r[1] = st[1]; r[2] = st[2];
                r[3] = st[3]; r[4] = st[4]; r[5] = st[5]; r[6] = st[6];
                r[7] = st[14] > 0 ? 0 : 1;
                rec_i++;
            }
            if (st[14] > 0) continue;
            do_step(&fc, pc, pn, nt, st, step, OR_SIM_MAX_STEPS, NULL);
        }
    }
    *fitness = st[15];
}

void FN(eval_prepared)(const R* pc, const R* pn, const R* mp, const int* nt, int pop,
                       const int* seeds, int nseeds, int vary, int max_steps, R* dist,
                       int* steps, int nthreads) {
    long nf = (long)pop * nseeds;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (long f = 0; f < nf; f++) {
        int p = (int)(f / nseeds), s = (int)(f % nseeds);
        int env_seed = (int)((uint32_t)seeds[s] + (vary ? (uint32_t)p * 7919u : 0u));
        int n = 0; R fit = 0;
        FN(fly)(pc + (size_t)p * OR_MAX_T * 4, pn + (size_t)p * OR_MAX_T * 4, nt[p],
                mp + (size_t)p * OR_MP_N, env_seed, max_steps, &fit, &n, NULL);
        dist[f] = fit;
        if (steps) steps[f] = n;
    }
}

void FN(eval_batch)(const float* genomes, int pop, const int* seeds, int nseeds, int vary,
                    int max_steps, R* dist, int* steps, int nthreads) {
    R* pc = (R*)malloc(sizeof(R) * (size_t)pop * OR_MAX_T * 4);
    R* pn = (R*)malloc(sizeof(R) * (size_t)pop * OR_MAX_T * 4);
    R* mp = (R*)malloc(sizeof(R) * (size_t)pop * OR_MP_N);
    int* nt = (int*)malloc(sizeof(int) * (size_t)pop);
    FN(prepare)(genomes, pop, pc, pn, mp, nt);
    FN(eval_prepared)(pc, pn, mp, nt, pop, seeds, nseeds, vary, max_steps, dist, steps, nthreads);
    free(pc); free(pn); free(mp); free(nt);
}
