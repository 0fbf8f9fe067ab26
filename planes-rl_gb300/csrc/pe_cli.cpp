// pe_cli.cpp -- `planes`: the reference's command line (src/main.cu:36-106) for the modes that
// run the fitness path: evolve, evaluate, select-best.  Same flags and defaults.  The video,
// STL and preset modes belong to the reference's renderer / exporters and are not part of this
// build.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <filesystem>
#include <string>
#include <vector>

#include "planes_eval.h"

static const char* opt(int argc, char** argv, const char* key, const char* dflt) {
    for (int i = 2; i < argc - 1; i++)
        if (!strcmp(argv[i], key)) return argv[i + 1];
    return dflt;
}

static int usage() {
    printf("usage: planes <evolve|evaluate|select-best> [opts]\n"
           "  evolve    --pop 4096 --gens 400 --seeds 8 --out out [--init out/pop.bin]\n"
           "            [--device 1 [--seed 42] [--polish-top 64 --polish-steps 8 --polish-lr 0.01]\n"
           "             [--audit 4096]]   device GA / hybrid search (pe_evolve)\n"
           "  evaluate  --best out/best.bin --n 512 --seed 9001 --o out/robustness.csv\n"
           "  select-best --pop-file out/archive.bin --n 8192 --seed 1900001 --out out/run\n");
    return 1;
}

static int report(int rc) {
    if (rc != PE_OK) fprintf(stderr, "planes: error %d: %s\n", rc, pe_last_error());
    return rc == PE_OK ? 0 : 1;
}

// evolve --device 1: the GA on the device (pe_evolve), optionally with Adam polish on the adjoint.
// Writes <out>/best.bin and <out>/history.csv (the host GA's columns plus device seconds).
static int evolve_device(int argc, char** argv) {
    if (opt(argc, argv, "--init", nullptr)) {
        fprintf(stderr, "planes: --init is supported by the host GA only (omit --device)\n");
        return 1;
    }
    pe_evolve_config c{};
    c.pop = atoi(opt(argc, argv, "--pop", "4096"));
    c.gens = atoi(opt(argc, argv, "--gens", "400"));
    c.nseeds = atoi(opt(argc, argv, "--seeds", "3"));
    c.seed = (unsigned)strtoul(opt(argc, argv, "--seed", "42"), nullptr, 10);
    c.max_steps = 7200;
    c.polish_top = atoi(opt(argc, argv, "--polish-top", "0"));
    c.polish_steps = atoi(opt(argc, argv, "--polish-steps", "8"));
    c.polish_lr = (float)atof(opt(argc, argv, "--polish-lr", "0.01"));
    c.polish_max_steps = 0;
    c.holdout = 128;  // the top 8 on 128 scenarios every generation, src/sim.cu:446-456
    c.holdout_base = 100003;
    c.audit = atoi(opt(argc, argv, "--audit", "0"));
    c.audit_base = 9001;
    const std::string out = opt(argc, argv, "--out", "out");
    std::error_code ec;
    std::filesystem::create_directories(out, ec);
    pe_engine* e = nullptr;
    if (int rc = pe_engine_create(0, &e)) return report(rc);
    std::vector<float> hist((size_t)(c.gens > 0 ? c.gens : 1) * 5);
    pe_evolve_result r{};
    int rc = pe_evolve(e, &c, hist.data(), &r);
    pe_engine_destroy(e);
    if (rc != PE_OK) return report(rc);
    FILE* f = fopen((out + "/history.csv").c_str(), "w");
    if (!f) { fprintf(stderr, "planes: cannot write %s/history.csv\n", out.c_str()); return 1; }
    fprintf(f, "gen,train_best,holdout128,mean,p90,gpu_s\n");
    for (int g = 0; g < c.gens; g++) {
        const float* h = &hist[(size_t)g * 5];
        fprintf(f, "%d,%.3f,%.3f,%.3f,%.3f,%.4f\n", g, h[0], h[1], h[2], h[3], h[4]);
        if (g % 10 == 0 || g == c.gens - 1)
            printf("gen %4d train %7.2fm holdout %7.2fm mean %7.2fm p90 %7.2fm\n", g, h[0], h[1], h[2], h[3]);
    }
    fclose(f);
    if (int rc2 = pe_save_best((out + "/best.bin").c_str(), r.best_genome)) return report(rc2);
    printf("best holdout score: %.2fm (generation %d, saved %s/best.bin), %.2f GPU s, %d gradient calls\n",
           r.best_holdout, r.best_gen, out.c_str(), r.gpu_seconds, r.grad_calls);
    if (c.audit > 0) printf("audit on %d scenarios: %.2fm\n", c.audit, r.audit_score);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return usage();
    const char* mode = argv[1];
    if (!strcmp(mode, "evolve") && atoi(opt(argc, argv, "--device", "0"))) return evolve_device(argc, argv);
    if (!strcmp(mode, "evolve")) {
        return report(pe_run_ga(atoi(opt(argc, argv, "--pop", "4096")), atoi(opt(argc, argv, "--gens", "400")),
                                atoi(opt(argc, argv, "--seeds", "3")), opt(argc, argv, "--out", "out"),
                                opt(argc, argv, "--init", nullptr)));
    }
    if (!strcmp(mode, "evaluate")) {
        float g[PE_GENOME_FLOATS];
        const char* path = opt(argc, argv, "--best", "out/best.bin");
        if (pe_load_best(path, g) != PE_OK) {
            fprintf(stderr, "missing %s\n", path);
            return 1;
        }
        return report(pe_evaluate_design(g, atoi(opt(argc, argv, "--n", "512")), atoi(opt(argc, argv, "--seed", "9001")),
                                         opt(argc, argv, "--o", "out/robustness.csv"), nullptr));
    }
    if (!strcmp(mode, "select-best")) {
        const char* path = opt(argc, argv, "--pop-file", "out/archive.bin");
        int n = 0;
        if (pe_load_genomes(path, nullptr, 0, &n) != PE_OK) {
            fprintf(stderr, "missing %s\n", path);
            return 1;
        }
        std::vector<float> gs((size_t)n * PE_GENOME_FLOATS);
        if (pe_load_genomes(path, gs.data(), n, &n) != PE_OK) {
            fprintf(stderr, "truncated %s\n", path);
            return 1;
        }
        return report(pe_select_finalist(gs.data(), n, atoi(opt(argc, argv, "--n", "8192")),
                                         atoi(opt(argc, argv, "--seed", "1900001")), opt(argc, argv, "--out", "out"),
                                         nullptr));
    }
    static const char* other[] = {"showcase", "hero", "robust-video", "evolution-video", "turntable", "stl",
                                  "inspect", "presets"};
    for (const char* o : other)
        if (!strcmp(mode, o)) {
            fprintf(stderr, "planes: mode %s belongs to the renderer / exporters, which are outside the fitness-evaluation path and not provided\n", mode);
            return 1;
        }
    fprintf(stderr, "unknown mode %s\n", mode);
    return 1;
}
