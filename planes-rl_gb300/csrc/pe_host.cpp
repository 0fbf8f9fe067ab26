// pe_host.cpp -- host-side parts of the evolve/evaluate call surface: genome draw and clamp,
// the best.bin / pop.bin formats (src/sim.cu:315-338, src/main.cu:22-34).
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <string>
#include <vector>

#include "planes_eval.h"

namespace {

// Genome clamp bounds in gene order (src/common.h:98-103).
const float kLo[PE_GENOME_FLOATS] = {
    0.12f, 0.05f, 0.04f, 0.00f, -0.30f, -1.20f, 0.45f, -0.04f, -0.06f, -0.20f, -0.20f, 0.0f,
    0.005f, 0.000f, 0.50f, 0.06f, 0.004f, 0.12f, 0.00f, 0.12f, 0.10f, -0.16f, -0.80f, -0.80f,
    -0.65f, -0.65f, 0.00f, 0.00f, 0.10f, 0.15f, -0.40f, 0.15f, -0.50f, 0.00f, -0.25f};
const float kHi[PE_GENOME_FLOATS] = {
    0.25f, 0.20f, 1.00f, 0.90f, 0.60f, 1.20f, 0.90f, 0.10f, 0.06f, 0.08f, 0.20f, 1.5f,
    0.050f, 0.060f, 1.00f, 0.30f, 0.065f, 0.65f, 0.85f, 0.65f, 0.45f, 0.16f, 0.80f, 0.80f,
    1.00f, 1.00f, 1.00f, 0.75f, 1.00f, 1.00f, 1.00f, 1.00f, 0.50f, 1.00f, 0.80f};

inline void gset(float* g, int i, float v) { g[i] = fminf(kHi[i], fmaxf(kLo[i], v)); }

}  // namespace

namespace pe {
void set_last_error(const char* msg);  // pe_api.cu
}

namespace {
// The message pe_last_error() returns, and PE_EINVAL.
int host_fail(const char* msg) {
    pe::set_last_error(msg);
    return PE_EINVAL;
}
}  // namespace

extern "C" {

int pe_genome_bounds(float* lo, float* hi) {
    if (!lo || !hi) return PE_EINVAL;
    memcpy(lo, kLo, sizeof kLo);
    memcpy(hi, kHi, sizeof kHi);
    return PE_OK;
}

// n genomes drawn as the reference's grand() does from std::mt19937(seed): gene i =
// clamp(G_LO[i] + u * (G_HI[i] - G_LO[i])), u from uniform_real_distribution<float>(0, 1).
int pe_random_genomes(unsigned seed, int n, float* h_out) {
    if (n < 0 || (n > 0 && !h_out)) return PE_EINVAL;
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> u(0, 1);
    for (int k = 0; k < n; k++)
        for (int i = 0; i < PE_GENOME_FLOATS; i++)
            gset(h_out + (size_t)k * PE_GENOME_FLOATS, i, kLo[i] + u(rng) * (kHi[i] - kLo[i]));
    return PE_OK;
}

// Clamp genomes to the bounds (the reference's sanitize(), applied to warm starts).
int pe_sanitize_genomes(float* h_genomes, int n) {
    if (n < 0 || (n > 0 && !h_genomes)) return PE_EINVAL;
    for (int k = 0; k < n; k++)
        for (int i = 0; i < PE_GENOME_FLOATS; i++) {
            float* g = h_genomes + (size_t)k * PE_GENOME_FLOATS;
            gset(g, i, g[i]);
        }
    return PE_OK;
}

// best.bin: one raw 140-byte genome.
int pe_save_best(const char* path, const float* genome) {
    if (!path || !genome) return host_fail("pe_save_best: NULL path or genome");
    FILE* f = fopen(path, "wb");
    if (!f) return host_fail("cannot create best-genome file");
    size_t w = fwrite(genome, sizeof(float), PE_GENOME_FLOATS, f);
    fclose(f);
    return w == PE_GENOME_FLOATS ? PE_OK : host_fail("short write of best-genome file");
}

int pe_load_best(const char* path, float* genome) {
    if (!path || !genome) return host_fail("pe_load_best: NULL path or genome");
    FILE* f = fopen(path, "rb");
    if (!f) return host_fail("cannot open best-genome file");
    size_t r = fread(genome, sizeof(float), PE_GENOME_FLOATS, f);
    fclose(f);
    return r == PE_GENOME_FLOATS ? PE_OK : host_fail("best-genome file is shorter than one genome (140 bytes)");
}

// pop.bin / archive.bin: int32 n, then n genomes.
int pe_save_genomes(const char* path, const float* genomes, int n) {
    if (!path || n < 0 || (n > 0 && !genomes)) return host_fail("pe_save_genomes: NULL path or genomes, or n < 0");
    FILE* f = fopen(path, "wb");
    if (!f) return host_fail("cannot create genome file");
    size_t w = fwrite(&n, 4, 1, f);
    w += fwrite(genomes, sizeof(float) * PE_GENOME_FLOATS, (size_t)n, f);
    fclose(f);
    return w == (size_t)n + 1 ? PE_OK : host_fail("short write of genome file");
}

// Reads up to `cap` genomes; *n_out = count in the file.  A file shorter than its header
// claims is an error (the reference reads it without a check, src/main.cu:28-34).
int pe_load_genomes(const char* path, float* genomes, int cap, int* n_out) {
    if (!path || !n_out || cap < 0) return host_fail("pe_load_genomes: NULL path or count, or negative cap");
    FILE* f = fopen(path, "rb");
    if (!f) return host_fail("cannot open genome file");
    int n = 0;
    if (fread(&n, 4, 1, f) != 1 || n < 0) { fclose(f); return host_fail("genome file has no valid count"); }
    *n_out = n;
    int k = std::min(n, cap);
    size_t r = k > 0 && genomes ? fread(genomes, sizeof(float) * PE_GENOME_FLOATS, (size_t)k, f) : (size_t)k;
    fclose(f);
    return r == (size_t)k ? PE_OK : host_fail("genome file is truncated: fewer genomes than its count");
}

}  // extern "C"
