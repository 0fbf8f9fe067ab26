// sim_gb300.cpp -- the reference-side binding of this library: drop-in definitions of the four
// functions of the reference's evaluation boundary (src/sim.h:9-13), replacing their bodies in
// src/sim.cu:214-248.  A maintainer compiles this file into the reference's build in place of those
// definitions and links -Lplanes-rl_gb300/lib -lplanes_gb300; the callers (run_ga, evaluate_design,
// select_finalist, record_flights) stay unchanged.
//
// Semantics kept: Genome is 35 floats (src/common.h:61-97), d_fitness[p] flies under
// seed + vary_scenarios * p * 7919, gpu_sim returns after the flights completed, oversize meshes
// score -100, d_rec / spread record poses in the reference's float8 layout.  Errors: the library
// returns status codes; this shim turns them into the reference's CK() behaviour (message, exit 1,
// src/sim.cu:11-12).
#include <cstdio>
#include <cstdlib>

#include "planes_eval.h"
#include "sim.h"

static_assert(sizeof(Genome) == PE_GENOME_FLOATS * sizeof(float), "Genome is 35 packed floats");
static_assert(sizeof(float8) == 8 * sizeof(float), "float8 is the pose record: pos xyz, q wxyz, alive");

static void check(int rc) {
    if (rc != PE_OK) {
        fprintf(stderr, "planes_eval: %s\n", pe_last_error());
        exit(1);
    }
}

void* panelbuf_alloc(int pop) {
    void* pb = nullptr;
    check(pe_panelbuf_alloc(pop, &pb));
    return pb;
}

void panelbuf_free(void* pb) { check(pe_panelbuf_free(pb)); }

void gpu_prepare(const Genome* d_gs, void* pb, int pop) {
    check(pe_prepare(reinterpret_cast<const float*>(d_gs), pb, pop, nullptr));
}

void gpu_sim(void* pb, int pop, int seed, float* d_fitness, float8* d_rec, int rec_every, int rec_cap,
             float spread, int vary_scenarios) {
    check(pe_sim(pb, pop, seed, d_fitness, reinterpret_cast<float*>(d_rec), rec_every, rec_cap, spread,
                 vary_scenarios, nullptr));
}
