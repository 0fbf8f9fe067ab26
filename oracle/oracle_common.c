/*
 * oracle_common.c -- precision-independent parts of the oracle (TEST INFRASTRUCTURE ONLY):
 * the tail-aware fitness reduction, the genome bounds and the seeded genome draw.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

/* Genome clamp bounds, gene order of the Genome struct (src/common.h:98-103). */
static const float LO[OR_GENOME_N] = {
    0.12f, 0.05f, 0.04f, 0.00f, -0.30f, -1.20f, 0.45f, -0.04f, -0.06f, -0.20f, -0.20f, 0.0f,
    0.005f, 0.000f, 0.50f, 0.06f, 0.004f, 0.12f, 0.00f, 0.12f, 0.10f, -0.16f, -0.80f, -0.80f,
    -0.65f, -0.65f, 0.00f, 0.00f, 0.10f, 0.15f, -0.40f, 0.15f, -0.50f, 0.00f, -0.25f};
static const float HI[OR_GENOME_N] = {
    0.25f, 0.20f, 1.00f, 0.90f, 0.60f, 1.20f, 0.90f, 0.10f, 0.06f, 0.08f, 0.20f, 1.5f,
    0.050f, 0.060f, 1.00f, 0.30f, 0.065f, 0.65f, 0.85f, 0.65f, 0.45f, 0.16f, 0.80f, 0.80f,
    1.00f, 1.00f, 1.00f, 0.75f, 1.00f, 1.00f, 1.00f, 1.00f, 0.50f, 1.00f, 0.80f};

void or_genome_bounds(float* lo, float* hi) {
    memcpy(lo, LO, sizeof LO);
    memcpy(hi, HI, sizeof HI);
}

static int cmp_f(const void* a, const void* b) {
    float x = *(const float*)a, y = *(const float*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* src/sim.cu:340-357 */
void or_robust_scores(const float* samples, int pop, int nseeds, float* scores) {
    float* row = (float*)malloc(sizeof(float) * (size_t)(nseeds > 0 ? nseeds : 1));
    int tail_n = (nseeds + 3) / 4;
    for (int i = 0; i < pop; i++) {
        float mean = 0;
        for (int s = 0; s < nseeds; s++) {
            row[s] = samples[(size_t)i * nseeds + s];
            mean += row[s] / (float)nseeds;
        }
        qsort(row, (size_t)nseeds, sizeof(float), cmp_f);
        float cvar = 0;
        for (int s = 0; s < tail_n; s++) cvar += row[s] / (float)tail_n;
        float a = 0.65f * mean, b = 0.25f * cvar, c = 0.10f * row[0];
        scores[i] = (a + b) + c;
    }
    free(row);
}

/* src/sim.cu:250-256 */
static float percentile_sorted(const float* s, int n, float q) {
    if (n <= 0) return 0;
    float x = q * (float)(n - 1);
    int a = (int)floorf(x), b = (int)ceilf(x);
    float t = x - (float)a;
    return s[a] * (1.0f - t) + s[b] * t;
}

/* src/sim.cu:291-309 */
void or_audit_stats(const float* dist, int n, float* out) {
    float* s = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    memcpy(s, dist, sizeof(float) * (size_t)n);
    qsort(s, (size_t)n, sizeof(float), cmp_f);
    float mean = 0, sq = 0;
    for (int i = 0; i < n; i++) {
        mean += s[i] / (float)n;
        sq += s[i] * s[i] / (float)n;
    }
    float sd = sqrtf(fmaxf(0.0f, sq - mean * mean));
    int tail_n = n / 10 > 1 ? n / 10 : 1, failures = 0;
    float cvar10 = 0;
    for (int i = 0; i < tail_n; i++) cvar10 += s[i] / (float)tail_n;
    for (int i = 0; i < n; i++)
        if (s[i] < 0.0f) failures++;
    out[0] = s[0];
    out[1] = percentile_sorted(s, n, .05f);
    out[2] = percentile_sorted(s, n, .10f);
    out[3] = percentile_sorted(s, n, .25f);
    out[4] = percentile_sorted(s, n, .50f);
    out[5] = mean;
    out[6] = sd;
    out[7] = percentile_sorted(s, n, .75f);
    out[8] = percentile_sorted(s, n, .90f);
    out[9] = percentile_sorted(s, n, .95f);
    out[10] = s[n - 1];
    out[11] = cvar10;
    out[12] = (float)failures;
    free(s);
}

/* MT19937 (Matsumoto & Nishimura 1998), seeded as std::mt19937(seed). */
typedef struct { uint32_t mt[624]; int idx; } mt_state;
static void mt_seed(mt_state* s, uint32_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
    s->idx = 624;
}
static uint32_t mt_next(mt_state* s) {
    if (s->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            uint32_t y = (s->mt[i] & 0x80000000u) | (s->mt[(i + 1) % 624] & 0x7fffffffu);
            s->mt[i] = s->mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        s->idx = 0;
    }
    uint32_t y = s->mt[s->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}
void or_mt19937_raw(uint32_t seed, int n, uint32_t* out) {
    mt_state s; mt_seed(&s, seed);
    for (int i = 0; i < n; i++) out[i] = mt_next(&s);
}
/* libstdc++ generate_canonical<float, 24> over a 32-bit engine: one draw, float(x) / 2^32,
 * with a result of 1 replaced by the largest float below 1. */
static float canonical_f(mt_state* s) {
    float x = (float)mt_next(s);
    float u = x / 4294967296.0f;
    if (u >= 1.0f) u = nextafterf(1.0f, 0.0f);
    return u;
}
/* src/sim.cu:316-321: gset(g, i, G_LO[i] + u * (G_HI[i] - G_LO[i])) */
void or_grand(uint32_t seed, int n, float* genomes) {
    mt_state s; mt_seed(&s, seed);
    for (int k = 0; k < n; k++)
        for (int i = 0; i < OR_GENOME_N; i++) {
            float u = canonical_f(&s);
            float v = LO[i] + u * (HI[i] - LO[i]);
            genomes[(size_t)k * OR_GENOME_N + i] = fminf(HI[i], fmaxf(LO[i], v));
        }
}
